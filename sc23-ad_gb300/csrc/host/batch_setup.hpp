// Host assembly of a batch of independent systems into block-diagonal level
// operators, so that one launch per operation serves every system.
//
// Each system keeps its own hierarchy, built exactly as intAMGflex builds it
// (INTAMG.hpp:149-245) with the multicolour smoother split; the batch only
// renumbers rows.  Systems have different depths D_s.  Level l of the batch
// holds the systems with D_s >= l: first those that smooth at level l
// (D_s > l), then those whose coarsest (LU) level is l.  Every batched integer
// operator carries the fractional bits of each row (its system's bits), so a
// row of the batch computes exactly what the same row of the system's own
// operator computes.
#pragma once
#include <cstdint>
#include <memory>
#include <functional>
#include <vector>

#include "amg_setup.hpp"
#include "csr.hpp"

namespace sagb {

// Block-diagonal integer CSR with per-row shifts.
struct BatchCsr {
    int n = 0, m = 0;
    std::vector<int> rptr, cind;
    std::vector<int32_t> val;
    std::vector<signed char> bit, dbit;  // per row (dbit: inverse-diagonal shift of LD rows)
    int64_t nnz() const { return rptr.empty() ? 0 : rptr[n]; }
};

struct BatchLevel {
    int n_all = 0;     // rows of the level vector
    int n_smooth = 0;  // rows of the systems that smooth here (a prefix)
    BatchCsr A;        // level operator over the smoothing prefix (A0 at level 0, C_A above)
    BatchCsr LD, U;    // multicolour SOR split over the smoothing prefix
    BatchCsr P;        // n_smooth x n_all(l+1): interpolation from level l+1
    BatchCsr R;        // n_all(l+1) x n_smooth: restriction to level l+1
    std::vector<int> colour_rows;  // smoothing rows grouped by colour
    std::vector<int> colour_ptr;   // colour k: colour_rows[colour_ptr[k] .. colour_ptr[k+1])
};

struct BatchLU {  // dense coarsest factors of one system (row-major, n x n)
    int sys = 0, level = 0, n = 0, offset = 0;  // rows [offset, offset+n) of that level's vector
    int bitL = 0, bitU = 0, dbitU = 0;
    std::vector<int32_t> L, U, dinv;
};

struct BatchHierarchy {
    int S = 0, Dmax = 0;
    std::vector<int> depth;                  // D_s
    std::vector<std::vector<int>> offset;    // offset[l][s]: first row of system s at level l (-1: absent)
    std::vector<BatchLevel> lv;              // l = 0 .. Dmax-1 (smoothing levels) plus the vector sizes of Dmax
    std::vector<int> n_level;                // rows of level l = 0 .. Dmax
    std::vector<std::vector<int>> row_sys;   // system of each row of level l = 0 .. Dmax
    std::vector<BatchLU> lu;
    BatchCsr A0;                             // == lv[0].A (fixed, 30 bits)
    CsrD Af;                                 // block-diagonal FP64 fine operator (refinement residual)
    std::vector<int> n_sys;                  // rows of each system
    std::vector<std::shared_ptr<RsChain>> chain;    // per system (for the FP64 rule V-cycle)
    std::vector<std::shared_ptr<CsrD>> A_sys;       // per system scaled fine matrix
    std::vector<std::shared_ptr<IntHierarchy>> hi;  // per system
    SmootherSpec sm;                                // the smoother every system was built with
};

// The same batch with every system's smoother split rebuilt for other colour
// caps (sm): the coarsening chains and scaled matrices are kept.
BatchHierarchy rebuild_batch_smoothers(const BatchHierarchy &old, const SmootherSpec &sm, int threads);

// The FP64 / FP32 sibling of a batch (dfAMG, INTAMG.hpp:13-134, per system):
// the same systems, coarsening chains, level order and row offsets as the
// integer batch it derives from, with the floating-point level operators
// (no row scaling, no quantisation), the multicolour SOR split of each level
// in the colours of that level's greedy colouring (the same cap), and dense
// coarsest LU factors.  LD rows hold the couplings to earlier colours, then
// the inverse diagonal last; the dense U holds the strict upper part and
// dinv the inverse diagonal (ltri / dutri::CSR<T>, ltri.hpp:19-54,
// dutri.hpp:19-55).
template <typename T>
struct BatchCsrT {
    int n = 0, m = 0;
    std::vector<int> rptr, cind;
    std::vector<T> val;
    int64_t nnz() const { return rptr.empty() ? 0 : rptr[n]; }
};

template <typename T>
struct BatchLevelT {
    BatchCsrT<T> A, LD, U, P, R;   // as BatchLevel
    std::vector<int> colour_rows;  // smoothing rows grouped by colour (rows ascending in a colour)
    std::vector<int> colour_ptr;
};

template <typename T>
struct BatchLUT {
    int sys = 0, level = 0, n = 0, offset = 0;
    std::vector<T> L, U, dinv;  // dense row-major strict parts, inverse diagonal
};

template <typename T>
struct BatchFp {
    std::vector<BatchLevelT<T>> lv;  // l = 0 .. Dmax-1 of the integer batch
    std::vector<BatchLUT<T>> lu;     // one per system
};

// Builds every system's dfAMG hierarchy on host threads from the batch's
// chains and scaled matrices, then assembles the block-diagonal levels.
template <typename T>
BatchFp<T> build_batch_fp(const BatchHierarchy &B, int threads);

// Build the hierarchies of all systems (threads over systems) and assemble the
// batch.  The systems must already be scaled (LMax1Scaling).  src[s] (optional)
// names the system whose matrix and hierarchy system s repeats (src[s] <= s),
// so copies of one matrix, e.g. solved with different fractional bits, share
// one setup.
// big_chain, when given, builds the Ruge-Stueben chain of every system with at
// least big_rows rows (on the calling thread, before the others start), e.g.
// on a GPU; it must return what rs_chain returns.
BatchHierarchy build_batch(const std::vector<CsrD> &systems, double theta, int max_levels, double omega,
                           int smooth_iter, int threads, const std::vector<int> &src = {}, int max_colours = 0,
                           int coarse_colours = 0, int coarse_size = 2000,
                           const std::function<RsChain(const CsrD &)> &big_chain = nullptr, int big_rows = 0);

}  // namespace sagb
