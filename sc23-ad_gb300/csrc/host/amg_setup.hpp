// Host AMG setup: Ruge-Stueben coarsening, interpolation, Galerkin products,
// smoother splits, the coarse LU factorisation and the fixed-point conversion
// rules.  The solve phase runs on the GPU; this part stays on the host (as in
// the reference, whose timer starts after setup, Work/main.cpp:167).
//
// Every floating-point result must equal the reference's bit for bit, because
// the integer operators are derived from these values by truncation.  The code
// therefore performs the same IEEE operations in the same order as the
// reference and must be compiled without FP contraction (-ffp-contract=off).
#pragma once
#include <algorithm>
#include <cstdint>
#include <vector>

#include "csr.hpp"

namespace sagb {

// ------------------------------------------------------------ host threads
// The setup spreads independent work (Galerkin columns, the levels' smoother
// splits and conversions) over host threads.  A caller that already runs
// setups on several threads holds a HostSerial in each worker, and the setup
// then stays on that thread.
struct HostSerial {
    HostSerial();
    ~HostSerial();
    HostSerial(const HostSerial &) = delete;
    HostSerial &operator=(const HostSerial &) = delete;
};
bool host_serial();

// ------------------------------------------------------------ conversion rules
int ceil_log2_int(int64_t k);
// CSRflex / ldtri::CSRflex rule (matrix/spmat.hpp:108, ldtri.hpp:144-145)
int flex_bit(double max_abs);
// ltri/dutri::CSRflex rule (ltri.hpp:106-108, dutri.hpp:120-125)
int while_bit(double max_abs);
// (int)(v * (1 << bit)) with x86 cvttsd2si semantics (truncation, INT_MIN when
// out of range) so that every host gives the same integers.
int32_t quantize(double v, int bit);
// Work/main.cpp:160: F = c_max/||b|| < 1 ? 29 : 31 - (ceil(log2(int(c_max/||b||)+1)) + 1)
int rule_frac_bits(double c_max, double nrm_b);

// ------------------------------------------------------------------ preprocessing
// CSRMat::LMax1Scaling (matrix/csrmat.hpp:70-80)
void lmax1_scaling(CsrD &A, double *b);

// ------------------------------------------------------------ one coarsening level
// The two sequential steps of the C/F splitting, also used by the GPU setup
// (which runs the rest of a level on the device):
//   first_pass (helper_multigrid.hpp:138-266), second_pass (378-417).
struct Pattern {  // CSR without values
    int n = 0;
    std::vector<int> rptr, cind;
};
void rs_first_pass(const CsrD &S, const Pattern &St, std::vector<int> &is_coarse);
void rs_second_pass(const CsrD &S, std::vector<int> &is_coarse);

// helper::multigrid::get_amg_set (helper/helper_multigrid.hpp:34-63):
// from A build the coarse operator CA = P^T A P, P (Intrpl) and R = P^T (Intrpl_t).
void rs_level(const CsrD &A, double theta, CsrD &CA, CsrD &P, CsrD &R);

// The level loop shared by dfAMG and intAMGflex (INTAMG.hpp:38-51, 162-195):
// levels are added while max_levels > depth and the last coarse size >
// coarse_size (the reference's 2000 by default).  With another coarse_size
// (not the reference's rule) the chain also ends when a step keeps more than
// 90 % of the rows.
struct RsChain {
    std::vector<CsrD> CA, P, R;  // unscaled, CA[i] = R[i] * A_i * P[i]
    int depth() const { return (int)CA.size(); }
};
RsChain rs_chain(const CsrD &A, double theta, int max_levels, int coarse_size = 2000);

// ---------------------------------------------------------------- smoother splits
// SOR ctor (smoother/stationary.hpp:195-231): LD = strict lower + diag/omega
// (diagonal last in the row), U = (1 - 1/omega) diag first, then strict upper.
void sor_split(const CsrD &A, double omega, CsrD &LD, CsrD &U);
// BlockSOR / BlockSORflex ctor (stationary.hpp:704-765, 929-988): nb contiguous
// blocks; in-block lower + diag/omega -> LD, the rest -> U (original order).
void block_sor_split(const CsrD &A, double omega, int nb, CsrD &LD, CsrD &U, std::vector<int> &bj);
// helper::matrix::extractLDinv (helper_matrix.hpp:634-664)
CsrD extract_ldinv(const CsrD &A);
// helper::matrix::extractL / extractDinvU (helper_matrix.hpp:606-632, 698-728)
CsrD extract_l(const CsrD &A);
CsrD extract_dinvu(const CsrD &A);
// helper::matrix::ilu (helper_matrix.hpp:978-1061): exact LU with fill, L and U
// in one CSR (unit L multipliers below the diagonal).
CsrD ilu_full(const CsrD &A);

// ------------------------------------------------------------------ quantisation
CsrI to_fixed(const CsrD &A, int bit);             // CSR<Fixed<bit>> (spmat.hpp:62-70)
CsrI to_flex(const CsrD &A);                       // CSRflex (spmat.hpp:96-121)
CsrI to_ldtri_flex(const CsrD &LDinv);             // ldtri::CSRflex on extractLDinv output
CsrI to_ltri_flex(const CsrD &L);                  // ltri::CSRflex on extractL output
CsrI to_dutri_flex(const CsrD &DinvU);             // dutri::CSRflex on extractDinvU output

// --------------------------------------------------------------------- hierarchies
struct SmootherSpec {
    int block = 0;       // 0: SOR, else BlockSOR with this many blocks
    double omega = 1.0;
    int iter = 1;
    int multicolor = 0;  // 1: SOR in colour order (the multicolour variant); 2: JacobiSORflex
    int max_colours = 0; // multicolour: at most this many colours (0: as many as a proper colouring needs)
    int coarse_colours = 0;  // multicolour: the cap below the finest level (0: max_colours)
    std::vector<int> level_caps;  // multicolour: a cap per level, the last for all deeper ones (overrides both)
    int cap(int level) const {
        if (!level_caps.empty()) return level_caps[std::min(level, (int)level_caps.size() - 1)];
        return level > 0 && coarse_colours > 0 ? coarse_colours : max_colours;
    }
};

// Greedy colouring, colour by colour, on the symmetrised pattern (the
// reference's coloring_greedy, Library/helper/helper_graph.hpp:191-219).
// Returns 0-based colours; *ncolors set.  With max_colours > 0 the colouring
// stops after that many colours and the remaining rows join the colour where
// they have the fewest neighbours (no longer a proper colouring: within a
// colour those couplings are then applied Jacobi-like through U).
std::vector<int> greedy_colouring(const CsrD &A, int *ncolors, int max_colours = 0);
// SOR split in colour order: LD = couplings to earlier colours + diag/omega
// (diagonal last), U = (1 - 1/omega) diag first + couplings to later colours.
// GS with this split is ldtri::MCCSRflex (ldtri.hpp:635-700) without renumbering.
void mc_sor_split(const CsrD &A, double omega, const std::vector<int> &colour, CsrD &LD, CsrD &U);
// JacobiSORflex (smoother/stationary.hpp:564-676): consecutive chunks of
// kJacobiSorChunk rows; LD holds a row's couplings to earlier chunks and
// diag/omega, U the (1 - 1/omega) diagonal and every coupling inside the
// chunk or to later ones, each in the row's own entry order (the reference's
// arrays entry for entry).  The chunks are the colours of the sweep
// (ldtri::MCCSRflex order): a chunk's rows read only earlier chunks.
constexpr int kJacobiSorChunk = 1200;
void jacobi_sor_split(const CsrD &A, double omega, CsrD &LD, CsrD &U, std::vector<int> &colour);

struct IntHierarchy {
    int depth = 0;
    int smooth_iter = 1;
    CsrI A0;                     // CSR<Fixed<30>> of the fine operator
    std::vector<CsrI> CA, P, R;  // C_A[depth-1], Intrpl[depth], Intrpl_t[depth]
    std::vector<CsrI> LD, U;     // smoother of level l, l = 0..depth-1
    std::vector<std::vector<int>> bj;
    std::vector<std::vector<int>> colour;  // multicolour variant: 0-based colour per row
    CsrI LUL, LUU;
};

template <typename T>
struct FpHierarchy {
    int depth = 0;
    int smooth_iter = 1;
    CsrT<T> A0;
    std::vector<CsrT<T>> CA, P, R, LD, U;
    std::vector<std::vector<int>> bj;
    std::vector<std::vector<int>> colour;
    CsrT<T> LUL, LUU;
};

// intAMGflex ctor (INTAMG.hpp:149-245) on an already scaled fine matrix.
IntHierarchy build_int_hierarchy(const CsrD &A, const RsChain &chain, const SmootherSpec &sm);
// dfAMG ctor (INTAMG.hpp:25-84) in FP64 / FP32.
FpHierarchy<double> build_f64_hierarchy(const CsrD &A, const RsChain &chain, const SmootherSpec &sm);
FpHierarchy<float> build_f32_hierarchy(const CsrD &A, const RsChain &chain, const SmootherSpec &sm);

}  // namespace sagb
