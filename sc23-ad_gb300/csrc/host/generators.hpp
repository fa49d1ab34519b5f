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

// io::ReadMM(path, true, false) (Library/io/mm.hpp:24-98); throws SetupError.
// The entry lines are parsed on host threads (std::from_chars where it reads
// the whole token, strtol / strtod otherwise: the same numbers as the
// reference's strtod), then sorted with the reference's quicksort.
CsrD read_matrix_market(const char *path);

// A binary CSR file (rptr, cind, val after a header that records the size and
// modification time of the Matrix Market file it was read from).
void write_csr_binary(const CsrD &A, const char *path, int64_t src_size = -1, int64_t src_mtime_ns = -1);
bool read_csr_binary(const char *path, CsrD &A, int64_t *src_size, int64_t *src_mtime_ns);  // false: absent/invalid
// the cache when it was written from this very file (same size and mtime),
// else read_matrix_market, then the cache is (re)written
CsrD read_matrix_market_cached(const char *mm_path, const char *cache_path);

}  // namespace sagb
