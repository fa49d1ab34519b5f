// Level scheduling of sparse triangular sweeps.
//
// A sweep out_i = f(in_i, out_j for j in deps(i)) is run on the GPU in an order
// that respects the reference's sequential dependency order: each row waits
// only for the rows it reads, so the integer results are identical to the
// sequential loop (int64 sums are order independent).  Rows are grouped by
// level (level(i) = 1 + max level of its dependencies) and then cut into
// chunks that the kernel claims in order:
//   * a chunk is a contiguous range of level-ordered positions;
//   * a chunk either covers part of one level, or a run of consecutive small
//     levels (processed with a block barrier between them).
// Every dependency of a chunk lies in an earlier chunk or in an earlier level of
// the same chunk, so claiming chunks in increasing order cannot deadlock.
#pragma once
#include <cstdint>
#include <vector>

#include "csr.hpp"

namespace sagb {

enum TriKind : int {
    TRI_LD = 0,  // forward, off-diagonal entries then D^-1 last in the row (ldtri)
    TRI_L = 1,   // forward, unit diagonal, strictly lower entries (ltri)
    TRI_DU = 2,  // backward, D^-1 first then strictly upper entries (dutri)
};

struct TriSchedule {
    int n = 0, kind = TRI_LD;
    int nlev = 0;
    std::vector<int> perm;                // position -> row
    std::vector<int> prp, pci;            // off-diagonal entries in position order
    std::vector<int> diag_src;            // position -> index of D^-1 in the source CSR (or -1)
    std::vector<int> src_idx;             // off-diagonal entry -> index in the source CSR
    std::vector<int> chunk_lv;            // chunk c covers sub-levels [chunk_lv[c], chunk_lv[c+1])
    std::vector<int> sub_bound;           // sub-level s covers positions [sub_bound[s], sub_bound[s+1])
    std::vector<int> lvl_ptr;             // level l covers positions [lvl_ptr[l], lvl_ptr[l+1])
    std::vector<int> sub_level;           // level of each sub-level
    int max_level_rows = 0;
    int nchunks() const { return (int)chunk_lv.size() - 1; }
};

// rows_per_chunk: maximum rows of one chunk; also the threshold below which a
// level is merged with its neighbours into a run chunk.
// level_hint (optional): a level per row in which every dependency has a lower
// level (the colour index of a multicolour sweep); the DAG levels otherwise.
TriSchedule build_tri_schedule(const int *rptr, const int *cind, int n, int kind, int rows_per_chunk,
                               int max_run_levels, const int *level_hint = nullptr);

}  // namespace sagb
