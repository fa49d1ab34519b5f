#include "batch_setup.hpp"

#include <algorithm>
#include <atomic>
#include <memory>
#include <thread>

namespace sagb {

// append rows of a system block with row/column offsets and the block's shifts;
// drop_zeros leaves out stored zero values (they add nothing to an integer row
// sum: SOR's U holds (1 - 1/omega) d = 0 first in every row at omega = 1)
static void append_block(BatchCsr &B, const CsrI &M, int col_off, int bit, int dbit, bool drop_zeros = false) {
    for (int i = 0; i < M.n; i++) {
        for (int j = M.rptr[i]; j < M.rptr[i + 1]; j++) {
            if (drop_zeros && M.val[j] == 0) continue;
            B.cind.push_back(M.cind[j] + col_off);
            B.val.push_back(M.val[j]);
        }
        B.rptr.push_back((int)B.cind.size());
        B.bit.push_back((signed char)bit);
        B.dbit.push_back((signed char)dbit);
    }
    B.n += M.n;
}

static void start(BatchCsr &B, int m) {
    B = BatchCsr();
    B.m = m;
    B.rptr.push_back(0);
}

static int level_size(const IntHierarchy &h, int l) { return l == 0 ? h.A0.n : h.R[l - 1].n; }

static void assemble_batch(BatchHierarchy &B);

BatchHierarchy build_batch(const std::vector<CsrD> &systems, double theta, int max_levels, double omega,
                           int smooth_iter, int threads, const std::vector<int> &src_in, int max_colours,
                           int coarse_colours, int coarse_size, const std::function<RsChain(const CsrD &)> &big_chain, int big_rows) {
    BatchHierarchy B;
    const int S = (int)systems.size();
    if (S == 0) throw SetupError{"empty batch"};
    std::vector<int> src(S);
    for (int s = 0; s < S; s++) {
        src[s] = src_in.empty() ? s : src_in[s];
        if (src[s] < 0 || src[s] > s || (src[s] != s && src[src[s]] != src[s]))
            throw SetupError{"invalid repeated-system index"};
    }
    B.S = S;
    B.chain.resize(S);
    B.hi.resize(S);
    B.A_sys.resize(S);
    B.depth.resize(S);
    B.n_sys.resize(S);
    // ---- per-system hierarchies (independent; threads over systems)
    SmootherSpec sm;
    sm.block = 0;
    sm.omega = omega;
    sm.iter = smooth_iter;
    sm.multicolor = 1;
    sm.max_colours = max_colours;
    sm.coarse_colours = coarse_colours;
    B.sm = sm;
    if (big_chain)
        for (int s = 0; s < S; s++)
            if (src[s] == s && systems[s].n >= big_rows)
                B.chain[s] = std::make_shared<RsChain>(big_chain(systems[s]));
    std::atomic<int> next{0};
    std::vector<std::string> errs(S);
    const int T = std::max(1, std::min(threads, S));
    auto work = [&]() {
        // several systems at once: each worker builds its systems alone
        std::unique_ptr<HostSerial> serial(T > 1 ? new HostSerial() : nullptr);
        for (;;) {
            const int s = next.fetch_add(1);
            if (s >= S) return;
            if (src[s] != s) continue;  // a copy: shares the hierarchy below
            try {
                B.A_sys[s] = std::make_shared<CsrD>(systems[s]);
                if (!B.chain[s])
                    B.chain[s] = std::make_shared<RsChain>(rs_chain(systems[s], theta, max_levels, coarse_size));
                B.hi[s] = std::make_shared<IntHierarchy>(build_int_hierarchy(systems[s], *B.chain[s], sm));
            } catch (const SetupError &e) {
                errs[s] = e.msg;
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < T; t++) pool.emplace_back(work);
    work();
    for (auto &t : pool) t.join();
    for (int s = 0; s < S; s++)
        if (!errs[s].empty()) throw SetupError{"system " + std::to_string(s) + ": " + errs[s]};
    for (int s = 0; s < S; s++)
        if (src[s] != s) {
            B.A_sys[s] = B.A_sys[src[s]];
            B.chain[s] = B.chain[src[s]];
            B.hi[s] = B.hi[src[s]];
        }
    assemble_batch(B);
    return B;
}

BatchHierarchy rebuild_batch_smoothers(const BatchHierarchy &old, const SmootherSpec &sm, int threads) {
    BatchHierarchy B;
    const int S = old.S;
    B.S = S;
    B.chain = old.chain;
    B.A_sys = old.A_sys;
    B.hi.resize(S);
    B.depth.resize(S);
    B.n_sys.resize(S);
    B.sm = sm;
    // systems that shared a hierarchy keep sharing one
    std::vector<int> src(S);
    for (int s = 0; s < S; s++) {
        src[s] = s;
        for (int t = 0; t < s; t++)
            if (old.hi[t] == old.hi[s]) {
                src[s] = t;
                break;
            }
    }
    std::atomic<int> next{0};
    std::vector<std::string> errs(S);
    const int T = std::max(1, std::min(threads, S));
    auto work = [&]() {
        std::unique_ptr<HostSerial> serial(T > 1 ? new HostSerial() : nullptr);
        for (;;) {
            const int s = next.fetch_add(1);
            if (s >= S) return;
            if (src[s] != s) continue;
            try {
                B.hi[s] = std::make_shared<IntHierarchy>(build_int_hierarchy(*B.A_sys[s], *B.chain[s], sm));
            } catch (const SetupError &e) {
                errs[s] = e.msg;
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < T; t++) pool.emplace_back(work);
    work();
    for (auto &t : pool) t.join();
    for (int s = 0; s < S; s++)
        if (!errs[s].empty()) throw SetupError{"system " + std::to_string(s) + ": " + errs[s]};
    for (int s = 0; s < S; s++) B.hi[s] = B.hi[src[s]];
    assemble_batch(B);
    return B;
}

// level order, offsets and the block-diagonal operators of a batch whose
// per-system hierarchies (hi, A_sys, chain) are built
static void assemble_batch(BatchHierarchy &B) {
    const int S = B.S;
    int Dmax = 0;
    for (int s = 0; s < S; s++) {
        B.depth[s] = B.hi[s]->depth;
        B.n_sys[s] = B.A_sys[s]->n;
        Dmax = std::max(Dmax, B.depth[s]);
    }
    B.Dmax = Dmax;
    // ---- level orders and offsets: smoothing systems first, then LU systems
    B.offset.assign(Dmax + 1, std::vector<int>(S, -1));
    B.n_level.assign(Dmax + 1, 0);
    std::vector<std::vector<int>> order(Dmax + 1);
    for (int l = 0; l <= Dmax; l++) {
        for (int s = 0; s < S; s++)
            if (B.depth[s] > l) order[l].push_back(s);
        const int nsm = (int)order[l].size();
        for (int s = 0; s < S; s++)
            if (B.depth[s] == l) order[l].push_back(s);
        int off = 0, off_sm = 0;
        for (int k = 0; k < (int)order[l].size(); k++) {
            const int s = order[l][k];
            B.offset[l][s] = off;
            off += level_size(*B.hi[s], l);
            if (k < nsm) off_sm = off;
        }
        B.n_level[l] = off;
        B.row_sys.emplace_back(off, 0);
        for (int s : order[l])
            for (int i = 0; i < level_size(*B.hi[s], l); i++) B.row_sys[l][B.offset[l][s] + i] = s;
        if (l < Dmax) {
            B.lv.emplace_back();
            B.lv[l].n_all = off;
            B.lv[l].n_smooth = off_sm;
        }
    }
    // ---- batched operators of each smoothing level
    for (int l = 0; l < Dmax; l++) {
        BatchLevel &L = B.lv[l];
        start(L.A, L.n_smooth);
        start(L.LD, L.n_smooth);
        start(L.U, L.n_smooth);
        start(L.P, B.n_level[l + 1]);
        std::vector<int> ncol;
        for (int s : order[l]) {
            const IntHierarchy &h = *B.hi[s];
            const int off = B.offset[l][s];
            if (h.depth <= l) continue;  // LU system at this level
            const CsrI &A = l == 0 ? h.A0 : h.CA[l - 1];
            append_block(L.A, A, off, A.bit, 0);
            append_block(L.LD, h.LD[l], off, h.LD[l].bit, h.LD[l].dbit);
            append_block(L.U, h.U[l], off, h.U[l].bit, 0, true);
            append_block(L.P, h.P[l], B.offset[l + 1][s], h.P[l].bit, 0);
            const std::vector<int> &col = h.colour[l];
            int nc = 0;
            for (int c : col) nc = std::max(nc, c + 1);
            if ((int)ncol.size() < nc) ncol.resize(nc, 0);
            for (int c : col) ncol[c]++;
        }
        // restriction rows follow the order of level l+1
        start(L.R, L.n_smooth);
        for (int s : order[l + 1]) {
            const IntHierarchy &h = *B.hi[s];
            append_block(L.R, h.R[l], B.offset[l][s], h.R[l].bit, 0);
        }
        // colour schedule over the smoothing rows (rows ascending inside a colour)
        L.colour_ptr.assign(ncol.size() + 1, 0);
        for (size_t c = 0; c < ncol.size(); c++) L.colour_ptr[c + 1] = L.colour_ptr[c] + ncol[c];
        L.colour_rows.assign(L.n_smooth, 0);
        std::vector<int> fill(L.colour_ptr.begin(), L.colour_ptr.end() - 1);
        for (int s : order[l]) {
            const IntHierarchy &h = *B.hi[s];
            if (h.depth <= l) continue;
            const int off = B.offset[l][s];
            for (int i = 0; i < (int)h.colour[l].size(); i++) L.colour_rows[fill[h.colour[l][i]]++] = off + i;
        }
        for (size_t c = 0; c < ncol.size(); c++)
            std::sort(L.colour_rows.begin() + L.colour_ptr[c], L.colour_rows.begin() + L.colour_ptr[c + 1]);
    }
    B.A0 = B.lv[0].A;
    // ---- coarsest LU factors, dense
    for (int s = 0; s < S; s++) {
        const IntHierarchy &h = *B.hi[s];
        BatchLU lu;
        lu.sys = s;
        lu.level = h.depth;
        lu.n = h.LUL.n;
        lu.offset = B.offset[h.depth][s];
        lu.bitL = h.LUL.bit;
        lu.bitU = h.LUU.bit;
        lu.dbitU = h.LUU.dbit;
        const int n = lu.n;
        lu.L.assign((size_t)n * n, 0);
        lu.U.assign((size_t)n * n, 0);
        lu.dinv.assign(n, 0);
        for (int i = 0; i < n; i++) {
            for (int j = h.LUL.rptr[i]; j < h.LUL.rptr[i + 1]; j++) lu.L[(size_t)i * n + h.LUL.cind[j]] = h.LUL.val[j];
            if (h.LUU.rptr[i + 1] > h.LUU.rptr[i]) lu.dinv[i] = h.LUU.val[h.LUU.rptr[i]];
            for (int j = h.LUU.rptr[i] + 1; j < h.LUU.rptr[i + 1]; j++)
                lu.U[(size_t)i * n + h.LUU.cind[j]] = h.LUU.val[j];
        }
        B.lu.push_back(std::move(lu));
    }
    // ---- FP64 fine operator (refinement residual), block diagonal in level-0 order
    B.Af.n = B.Af.m = B.n_level[0];
    B.Af.rptr.assign(1, 0);
    for (int s : order[0]) {
        const CsrD &A = *B.A_sys[s];
        const int off = B.offset[0][s];
        for (int i = 0; i < A.n; i++) {
            for (int j = A.rptr[i]; j < A.rptr[i + 1]; j++) {
                B.Af.cind.push_back(A.cind[j] + off);
                B.Af.val.push_back(A.val[j]);
            }
            B.Af.rptr.push_back((int)B.Af.cind.size());
        }
    }
}

// ------------------------------------------------ floating-point sibling

template <typename T>
static void start_t(BatchCsrT<T> &B, int m) {
    B = BatchCsrT<T>();
    B.m = m;
    B.rptr.push_back(0);
}

template <typename T>
static void append_t(BatchCsrT<T> &B, const CsrT<T> &M, int col_off, bool drop_zeros = false) {
    for (int i = 0; i < M.n; i++) {
        for (int j = M.rptr[i]; j < M.rptr[i + 1]; j++) {
            if (drop_zeros && M.val[j] == T(0)) continue;  // U's (1 - 1/omega) d at omega = 1
            B.cind.push_back(M.cind[j] + col_off);
            B.val.push_back(M.val[j]);
        }
        B.rptr.push_back((int)B.cind.size());
    }
    B.n += M.n;
}

template <typename T>
static FpHierarchy<T> fp_hierarchy(const CsrD &A, const RsChain &chain, const SmootherSpec &sm);
template <>
FpHierarchy<double> fp_hierarchy<double>(const CsrD &A, const RsChain &chain, const SmootherSpec &sm) {
    return build_f64_hierarchy(A, chain, sm);
}
template <>
FpHierarchy<float> fp_hierarchy<float>(const CsrD &A, const RsChain &chain, const SmootherSpec &sm) {
    return build_f32_hierarchy(A, chain, sm);
}

template <typename T>
BatchFp<T> build_batch_fp(const BatchHierarchy &B, int threads) {
    const int S = B.S, Dmax = B.Dmax;
    // per-system hierarchies; systems that repeat another share its hierarchy
    std::vector<std::shared_ptr<FpHierarchy<T>>> hs(S);
    std::vector<int> src(S);
    for (int s = 0; s < S; s++) {
        src[s] = s;
        for (int t = 0; t < s; t++)
            if (B.hi[t] == B.hi[s]) {
                src[s] = t;
                break;
            }
    }
    std::atomic<int> next{0};
    std::vector<std::string> errs(S);
    const int T_ = std::max(1, std::min(threads > 0 ? threads : (int)std::thread::hardware_concurrency(), S));
    auto work = [&]() {
        std::unique_ptr<HostSerial> serial(T_ > 1 ? new HostSerial() : nullptr);
        for (;;) {
            const int s = next.fetch_add(1);
            if (s >= S) return;
            if (src[s] != s) continue;
            try {
                hs[s] = std::make_shared<FpHierarchy<T>>(fp_hierarchy<T>(*B.A_sys[s], *B.chain[s], B.sm));
            } catch (const SetupError &e) {
                errs[s] = e.msg;
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < T_; t++) pool.emplace_back(work);
    work();
    for (auto &t : pool) t.join();
    for (int s = 0; s < S; s++)
        if (!errs[s].empty()) throw SetupError{"system " + std::to_string(s) + ": " + errs[s]};
    for (int s = 0; s < S; s++) hs[s] = hs[src[s]];
    // the integer batch's level order: smoothing systems first, then LU systems
    std::vector<std::vector<int>> order(Dmax + 1);
    for (int l = 0; l <= Dmax; l++) {
        for (int s = 0; s < S; s++)
            if (B.depth[s] > l) order[l].push_back(s);
        for (int s = 0; s < S; s++)
            if (B.depth[s] == l) order[l].push_back(s);
    }
    BatchFp<T> F;
    F.lv.resize(Dmax);
    for (int l = 0; l < Dmax; l++) {
        BatchLevelT<T> &L = F.lv[l];
        const int n_smooth = B.lv[l].n_smooth;
        start_t(L.A, n_smooth);
        start_t(L.LD, n_smooth);
        start_t(L.U, n_smooth);
        start_t(L.P, B.n_level[l + 1]);
        std::vector<int> ncol;
        for (int s : order[l]) {
            const FpHierarchy<T> &h = *hs[s];
            if (h.depth != B.depth[s]) throw SetupError{"FP hierarchy depth differs from the integer batch's"};
            if (h.depth <= l) continue;
            const int off = B.offset[l][s];
            append_t(L.A, l == 0 ? h.A0 : h.CA[l - 1], off);
            append_t(L.LD, h.LD[l], off);
            append_t(L.U, h.U[l], off, true);
            append_t(L.P, h.P[l], B.offset[l + 1][s]);
            int nc = 0;
            for (int c : h.colour[l]) nc = std::max(nc, c + 1);
            if ((int)ncol.size() < nc) ncol.resize(nc, 0);
            for (int c : h.colour[l]) ncol[c]++;
        }
        start_t(L.R, n_smooth);
        for (int s : order[l + 1]) append_t(L.R, hs[s]->R[l], B.offset[l][s]);
        L.colour_ptr.assign(ncol.size() + 1, 0);
        for (size_t c = 0; c < ncol.size(); c++) L.colour_ptr[c + 1] = L.colour_ptr[c] + ncol[c];
        L.colour_rows.assign(n_smooth, 0);
        std::vector<int> fill(L.colour_ptr.begin(), L.colour_ptr.end() - 1);
        for (int s : order[l]) {
            const FpHierarchy<T> &h = *hs[s];
            if (h.depth <= l) continue;
            const int off = B.offset[l][s];
            for (int i = 0; i < (int)h.colour[l].size(); i++) L.colour_rows[fill[h.colour[l][i]]++] = off + i;
        }
        for (size_t c = 0; c < ncol.size(); c++)
            std::sort(L.colour_rows.begin() + L.colour_ptr[c], L.colour_rows.begin() + L.colour_ptr[c + 1]);
    }
    for (int s = 0; s < S; s++) {
        const FpHierarchy<T> &h = *hs[s];
        BatchLUT<T> lu;
        lu.sys = s;
        lu.level = h.depth;
        lu.n = h.LUL.n;
        lu.offset = B.offset[h.depth][s];
        const int n = lu.n;
        lu.L.assign((size_t)n * n, T(0));
        lu.U.assign((size_t)n * n, T(0));
        lu.dinv.assign(n, T(0));
        for (int i = 0; i < n; i++) {
            for (int j = h.LUL.rptr[i]; j < h.LUL.rptr[i + 1]; j++) lu.L[(size_t)i * n + h.LUL.cind[j]] = h.LUL.val[j];
            if (h.LUU.rptr[i + 1] > h.LUU.rptr[i]) lu.dinv[i] = h.LUU.val[h.LUU.rptr[i]];
            for (int j = h.LUU.rptr[i] + 1; j < h.LUU.rptr[i + 1]; j++)
                lu.U[(size_t)i * n + h.LUU.cind[j]] = h.LUU.val[j];
        }
        F.lu.push_back(std::move(lu));
    }
    return F;
}

template BatchFp<double> build_batch_fp<double>(const BatchHierarchy &, int);
template BatchFp<float> build_batch_fp<float>(const BatchHierarchy &, int);

}  // namespace sagb
