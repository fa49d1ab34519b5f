// Synthetic sparse systems (the reference's SuiteSparse inputs are not shipped).
// Rows in natural order (x fastest), columns sorted, Dirichlet boundaries.
// tests/golden/gen_matrices.py is an independent numpy version of the same
// generators; the two are checked against each other.
#pragma once
#include <cstdint>
#include <vector>

#include "csr.hpp"

namespace sagb {

uint64_t splitmix64_at(uint64_t seed, uint64_t i);   // i-th output, i >= 1
double uniform01_at(uint64_t seed, uint64_t i);        // (z >> 11) * 2^-53

CsrD gen_poisson2d(int n);
CsrD gen_poisson3d(int n);
CsrD gen_aniso2d(int n, double eps);
CsrD gen_stencil27(int n, uint64_t seed);
CsrD gen_convdiff3d(int n, double pe);
CsrD gen_varcoef3d(int n, double sigma, uint64_t seed);
// x* ~ U[-1, 1] from splitmix64(seed), b = A x* in row order
void gen_rhs(const CsrD &A, uint64_t seed, double *xstar, double *b);

// io::ReadMM(path, true, false) (Library/io/mm.hpp:24-98); throws SetupError
CsrD read_matrix_market(const char *path);

}  // namespace sagb
