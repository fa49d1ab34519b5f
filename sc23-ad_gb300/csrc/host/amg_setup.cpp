// Host AMG setup (see amg_setup.hpp).  Reference paths are relative to the
// suzuki-hpc/SC23-AD tree.  The algorithms are restated step for step where the
// result depends on the order of operations (tie breaking in the coarsening,
// FP summation order); the data structures are our own (dense accumulators in
// place of the reference's realloc-per-column sparse vectors).
#include "amg_setup.hpp"
#include "sort.hpp"

#include <algorithm>
#include <atomic>
#include <exception>
#include <mutex>
#include <thread>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <numeric>
#include <utility>

namespace sagb {

static thread_local int tl_serial = 0;
HostSerial::HostSerial() { tl_serial++; }
HostSerial::~HostSerial() { tl_serial--; }
bool host_serial() { return tl_serial > 0; }

// f(0) .. f(n-1) on up to hardware_concurrency host threads; every task
// writes its own pre-sized slot, so results do not depend on the thread count
template <typename F>
static void parallel_tasks(int n, F &&f) {
    const int T = host_serial() ? 1 : std::min(n, (int)std::max(1u, std::thread::hardware_concurrency()));
    if (T <= 1) {
        for (int i = 0; i < n; i++) f(i);
        return;
    }
    std::atomic<int> next(0);
    std::exception_ptr first;
    std::mutex mu;
    std::vector<std::thread> pool;
    for (int t = 0; t < T; t++)
        pool.emplace_back([&] {
            HostSerial inner;
            for (int i; (i = next++) < n;) {
                try {
                    f(i);
                } catch (...) {
                    std::lock_guard<std::mutex> g(mu);
                    if (!first) first = std::current_exception();
                }
            }
        });
    for (auto &th : pool) th.join();
    if (first) std::rethrow_exception(first);
}


// ============================================================ conversion rules

int ceil_log2_int(int64_t k) {
    if (k <= 1) return 0;
    int b = 0;
    uint64_t v = (uint64_t)(k - 1);
    while (v) { b++; v >>= 1; }
    return b;
}

static int32_t cvtt_i32(double v) {  // x86 cvttsd2si: truncate, INT_MIN if out of range / NaN
    if (!(v > -2147483649.0 && v < 2147483648.0)) return INT32_MIN;
    return (int32_t)v;
}

int flex_bit(double max) {
    if (max < 1) return 30;
    return 32 - (ceil_log2_int((int64_t)cvtt_i32(max) + 1) + 1);
}

int while_bit(double max) {
    int bit = 0;
    while (bit < 30 && max * (double)(1 << bit) < (double)(1 << 30)) bit++;
    return bit;
}

int32_t quantize(double v, int bit) { return cvtt_i32(v * (double)(1 << bit)); }

int rule_frac_bits(double c_max, double nrm_b) {
    double q = c_max / nrm_b;
    if (q < 1) return 29;
    return 31 - (ceil_log2_int((int64_t)cvtt_i32(q) + 1) + 1);
}

// =============================================================== preprocessing

void lmax1_scaling(CsrD &A, double *b) {
    for (int i = 0; i < A.n; i++) {
        double mx = 0;
        for (int j = A.rptr[i]; j < A.rptr[i + 1]; j++)
            if (std::fabs(A.val[j]) > mx) mx = std::fabs(A.val[j]);
        for (int j = A.rptr[i]; j < A.rptr[i + 1]; j++) A.val[j] /= mx;
        if (b) b[i] /= mx;
    }
}

// ======================================================= Ruge-Stueben coarsening

// rows [0, n) in blocks of at least 16384 rows, one task per block
template <typename F>
static void row_blocks(int n, F &&f) {
    const int nb = std::max(1, std::min(64, n / 16384));
    parallel_tasks(nb, [&](int b) { f((int)((long long)n * b / nb), (int)((long long)n * (b + 1) / nb)); });
}

// get_strong_weak_set (helper_multigrid.hpp:67-108): off-diagonal a_ij is strong
// when |a_ij| >= theta * max_k!=i |a_ik|; everything else (diagonal included)
// goes to the weak set.  Rows are independent: counts, prefix sums, then the
// entries of each row in order (host threads over row blocks).
static void strong_weak(const CsrD &A, double theta, CsrD &S, CsrD &W) {
    const int N = A.n;
    S.n = W.n = S.m = W.m = N;
    S.rptr.assign(N + 1, 0);
    W.rptr.assign(N + 1, 0);
    std::vector<double> thr(N);
    row_blocks(N, [&](int i0, int i1) {
        for (int i = i0; i < i1; i++) {
            double mx = 0;
            for (int j = A.rptr[i]; j < A.rptr[i + 1]; j++)
                if (A.cind[j] != i && std::fabs(A.val[j]) > mx) mx = std::fabs(A.val[j]);
            thr[i] = theta * mx;
            int ns = 0;
            for (int j = A.rptr[i]; j < A.rptr[i + 1]; j++)
                if (A.cind[j] != i && std::fabs(A.val[j]) >= thr[i]) ns++;
            S.rptr[i + 1] = ns;
            W.rptr[i + 1] = A.rptr[i + 1] - A.rptr[i] - ns;
        }
    });
    for (int i = 0; i < N; i++) {
        S.rptr[i + 1] += S.rptr[i];
        W.rptr[i + 1] += W.rptr[i];
    }
    S.cind.resize(S.rptr[N]);
    S.val.resize(S.rptr[N]);
    W.cind.resize(W.rptr[N]);
    W.val.resize(W.rptr[N]);
    row_blocks(N, [&](int i0, int i1) {
        for (int i = i0; i < i1; i++) {
            int a = S.rptr[i], b = W.rptr[i];
            for (int j = A.rptr[i]; j < A.rptr[i + 1]; j++) {
                if (A.cind[j] != i && std::fabs(A.val[j]) >= thr[i]) {
                    S.cind[a] = A.cind[j];
                    S.val[a++] = A.val[j];
                } else {
                    W.cind[b] = A.cind[j];
                    W.val[b++] = A.val[j];
                }
            }
        }
    });
}

// get_influence_set (helper_multigrid.hpp:110-136): transpose of the pattern.
static Pattern transpose_pattern(const CsrD &S) {
    Pattern T;
    const int N = S.n;
    T.n = N;
    T.rptr.assign(N + 1, 0);
    for (int c : S.cind) T.rptr[c + 1]++;
    for (int i = 0; i < N; i++) T.rptr[i + 1] += T.rptr[i];
    T.cind.resize(S.cind.size());
    std::vector<int> fill(T.rptr.begin(), T.rptr.end() - 1);
    for (int i = 0; i < N; i++)
        for (int j = S.rptr[i]; j < S.rptr[i + 1]; j++) T.cind[fill[S.cind[j]]++] = i;
    return T;
}

// C/F state of a point that neither pass has classified yet
constexpr int kUnclassified = -1;

// Candidate coarse points of the first pass, ordered by weight: the number of
// not yet classified points that a candidate strongly influences.  The points
// sit in slots 0..N-1; all points of one weight fill one contiguous run of
// slots, the runs in decreasing weight, and inside a run the slot order breaks
// ties.  `head` is the slot of the candidate taken last: slots below it are
// spent.  lim[w] is the first slot after the runs of weight >= w.  A weight
// change moves a point across the boundary between two neighbouring runs by
// one exchange of slots, which keeps the order of everything else.
class CandidateRuns {
  public:
    // Ranks the points by weight (decreasing), then inside each weight by the
    // secondary key `tie` (increasing), with the reference's quicksort on the
    // same key arrays (helper_multigrid.hpp:138-175), so ties fall the same way.
    CandidateRuns(std::vector<int> weight, std::vector<int> second, std::vector<int> tie) : n_((int)weight.size()) {
        pt_.resize(n_);
        for (int i = 0; i < n_; i++) pt_[i] = i;
        wt_ = std::move(weight);
        if (n_ > 0) hoare_sort(0, n_ - 1, false, wt_.data(), second.data(), tie.data(), pt_.data());
        top_ = n_ > 0 ? wt_[0] : 0;
        std::vector<int> count(top_ + 1, 0);
        for (int w : wt_) count[w]++;
        lim_.assign(top_ + 2, 0);
        for (int w = top_; w >= 0; w--) lim_[w] = lim_[w + 1] + count[w];
        for (int w = top_; w >= 0; w--)
            if (lim_[w] - lim_[w + 1] > 1) hoare_sort(lim_[w + 1], lim_[w] - 1, true, tie.data(), pt_.data());
        slot_.resize(n_);
        for (int k = 0; k < n_; k++) slot_[pt_[k]] = k;
    }

    // the next candidate at or after `head` that `skip` does not reject; -1 at the end
    template <typename Skip>
    int take(Skip &&skip) {
        while (head_ < n_ && skip(pt_[head_])) head_++;
        return head_ < n_ ? pt_[head_] : -1;
    }
    void advance() { head_++; }

    // weight + 1: the point moves to the front of its run and joins the run above
    void raise(int point) {
        const int k = slot_[point];
        const int w = ++wt_[k];
        const int first_live = head_ + 1;
        int dest;
        if (w > top_) {  // a new heaviest run, just after the head
            top_ = w;
            lim_.resize(w + 2);
            lim_[w + 1] = first_live;
            lim_[w] = first_live + 1;
            dest = first_live;
        } else if (lim_[w] > first_live) {  // run w has live slots: append to it
            dest = lim_[w]++;
        } else {  // run w is spent: it restarts after the head
            dest = first_live;
            lim_[w] = first_live + 1;
        }
        exchange(k, dest);
    }

    // weight - 1 (not below 0): the point moves to the back of its run and joins the run below
    void lower(int point) {
        const int k = slot_[point];
        if (wt_[k] == 0) return;
        const int w = wt_[k]--;
        exchange(k, --lim_[w]);
    }

  private:
    void exchange(int a, int b) {
        std::swap(wt_[a], wt_[b]);
        std::swap(pt_[a], pt_[b]);
        slot_[pt_[a]] = a;
        slot_[pt_[b]] = b;
    }
    int n_, top_ = 0, head_ = 0;
    std::vector<int> pt_, wt_, slot_, lim_;
};

// first_pass (helper_multigrid.hpp:138-266): the candidate that influences the
// most unclassified points becomes coarse, the points it influences become
// fine, and the weights of the points around them are updated before the next
// candidate is taken.
void rs_first_pass(const CsrD &S, const Pattern &St, std::vector<int> &is_coarse) {
    const int N = S.n;
    is_coarse.assign(N, kUnclassified);
    std::vector<char> done(N, 0);
    std::vector<int> weight(N), depends(N), reach(N, 0);
    for (int i = 0; i < N; i++) {
        weight[i] = St.rptr[i + 1] - St.rptr[i];  // points that depend strongly on i
        depends[i] = S.rptr[i + 1] - S.rptr[i];
        if (weight[i] == 0 && depends[i] == 0) {  // isolated: fine from the start
            is_coarse[i] = 0;
            done[i] = 1;
        }
        for (int j = St.rptr[i]; j < St.rptr[i + 1]; j++) reach[i] += S.rptr[St.cind[j] + 1] - S.rptr[St.cind[j]];
    }
    CandidateRuns runs(std::move(weight), std::move(depends), std::move(reach));
    for (int c; (c = runs.take([&](int p) { return done[p] != 0; })) >= 0; runs.advance()) {
        done[c] = 1;
        is_coarse[c] = 1;
        for (int t = St.rptr[c]; t < St.rptr[c + 1]; t++) {
            const int f = St.cind[t];
            if (done[f]) continue;
            done[f] = 1;
            is_coarse[f] = 0;
            // every open point that f depends on now influences one more new fine point
            for (int u = S.rptr[f]; u < S.rptr[f + 1]; u++)
                if (!done[S.cind[u]]) runs.raise(S.cind[u]);
        }
        for (int u = S.rptr[c]; u < S.rptr[c + 1]; u++)
            if (!done[S.cind[u]]) runs.lower(S.cind[u]);
    }
}

// second_pass (helper_multigrid.hpp:378-417): a fine point with a strong fine
// neighbour that shares no strong coarse point with it becomes coarse.
void rs_second_pass(const CsrD &S, std::vector<int> &is_coarse) {
    const int N = S.n;
    for (int i = 0; i < N; i++) {
        if (is_coarse[i] == kUnclassified)  // the reference exits here (helper_multigrid.hpp:384)
            throw SetupError{"coarsening left point " + std::to_string(i) + " unclassified"};
        if (is_coarse[i]) continue;
        for (int j = S.rptr[i]; j < S.rptr[i + 1]; j++) {
            const int f = S.cind[j];
            if (is_coarse[f]) continue;
            bool shared = false;
            int a = S.rptr[i], b = S.rptr[f];
            while (a < S.rptr[i + 1] && b < S.rptr[f + 1]) {
                if (S.cind[b] < S.cind[a]) {
                    b++;
                } else if (S.cind[b] == S.cind[a]) {
                    if (is_coarse[S.cind[a]]) { shared = true; break; }
                    a++; b++;
                } else {
                    a++;
                }
            }
            if (shared) continue;
            is_coarse[i] = 1;
            break;
        }
    }
}

// sepalate_strong_to_coarse_fine + get_interpolation_matrix
// (helper_multigrid.hpp:419-532): direct interpolation
//   w_ij = -(a_ij + sum_m a_im a_mj / sum_{k in C_i} a_mk) / sum(weak row i)
// with the sum over strong fine neighbours m in row order.
static CsrD interpolation(const CsrD &A, const CsrD &S, const CsrD &W, const std::vector<int> &is_coarse) {
    const int N = A.n;
    std::vector<int> col(N, -1);
    int nc = 0;
    for (int i = 0; i < N; i++)
        if (is_coarse[i]) col[i] = nc++;
    CsrD P;
    P.n = N;
    P.m = nc;
    P.rptr.assign(N + 1, 0);
    // a coarse row has one entry, a fine row one per strong coarse neighbour
    for (int i = 0; i < N; i++) {
        int cnt = 1;
        if (!is_coarse[i]) {
            cnt = 0;
            for (int j = S.rptr[i]; j < S.rptr[i + 1]; j++) cnt += is_coarse[S.cind[j]] != 0;
        }
        P.rptr[i + 1] = P.rptr[i] + cnt;
    }
    P.cind.resize(P.rptr[N]);
    P.val.resize(P.rptr[N]);
    // rows on host threads; the "1 amk = 0" lines are counted per row and the
    // "2 amk = 0" stop recorded, then both reported in row order
    std::vector<int> warn(N, 0);
    std::vector<char> stop(N, 0);
    row_blocks(N, [&](int i0, int i1) {
        std::vector<int> cs, cf;  // column lists of C_Stg row i / DS_Stg row i
        std::vector<double> vs, vf;
        std::vector<double> amk_m, amj;
        for (int i = i0; i < i1; i++) {
            if (is_coarse[i]) {
                P.cind[P.rptr[i]] = col[i];
                P.val[P.rptr[i]] = 1;
                continue;
            }
            cs.clear(); vs.clear(); cf.clear(); vf.clear();
            for (int j = S.rptr[i]; j < S.rptr[i + 1]; j++) {
                if (is_coarse[S.cind[j]]) { cs.push_back(S.cind[j]); vs.push_back(S.val[j]); }
                else { cf.push_back(S.cind[j]); vf.push_back(S.val[j]); }
            }
            double deno = 0;
            for (int j = W.rptr[i]; j < W.rptr[i + 1]; j++) deno += W.val[j];
            const int ncs = (int)cs.size(), ncf = (int)cf.size();
            // sum_{k in C_i} a_mk for each strong fine m (merge in column order),
            // and a_mj for each (m, j) pair
            amk_m.assign(ncf, 0.0);
            amj.assign((size_t)ncf * ncs, 0.0);
            bool stopped = false;
            for (int q = 0; q < ncf && ncs > 0; q++) {
                const int mrow = cf[q];
                double amk = 0;
                bool hit = false;
                int a = A.rptr[mrow], k = 0;
                while (a < A.rptr[mrow + 1] && k < ncs) {
                    if (A.cind[a] < cs[k]) {
                        a++;
                    } else if (A.cind[a] == cs[k]) {
                        amk += A.val[a];
                        amj[(size_t)q * ncs + k] = A.val[a];
                        hit = true;
                        a++; k++;
                    } else {
                        k++;
                    }
                }
                if (amk == 0) {
                    if (hit) {
                        warn[i] += ncs;  // "1 amk = 0" once per (j, m) pair
                        amk = 0.00001;
                    } else {
                        stop[i] = 1;  // "2 amk = 0": the reference exits (helper_multigrid.hpp:518)
                        stopped = true;
                        break;
                    }
                }
                amk_m[q] = amk;
            }
            if (stopped) continue;
            for (int k = 0; k < ncs; k++) {
                double aij = vs[k];
                for (int q = 0; q < ncf; q++) aij += vf[q] * amj[(size_t)q * ncs + k] / amk_m[q];
                P.cind[P.rptr[i] + k] = col[cs[k]];
                P.val[P.rptr[i] + k] = -aij / deno;
            }
        }
    });
    for (int i = 0; i < N; i++) {
        for (int k = 0; k < warn[i]; k++) printf("1 amk = 0\n");
        if (stop[i]) {  // the reference prints this and exits (helper_multigrid.hpp:518)
            printf("2 amk = 0\n");
            fflush(stdout);
            throw SetupError{"interpolation: fine row " + std::to_string(i) +
                             " has a strong fine neighbour with no coupling to its coarse points (2 amk = 0)"};
        }
    }
    return P;
}

// transpose_interpolation_matrix (helper_multigrid.hpp:534-562)
static CsrD transpose(const CsrD &P) {
    CsrD R;
    R.n = P.m;
    R.m = P.n;
    R.rptr.assign(R.n + 1, 0);
    for (int c : P.cind) R.rptr[c + 1]++;
    for (int i = 0; i < R.n; i++) R.rptr[i + 1] += R.rptr[i];
    R.cind.resize(P.cind.size());
    R.val.resize(P.val.size());
    std::vector<int> fill(R.rptr.begin(), R.rptr.end() - 1);
    for (int i = 0; i < P.n; i++)
        for (int j = P.rptr[i]; j < P.rptr[i + 1]; j++) {
            int p = fill[P.cind[j]]++;
            R.cind[p] = i;
            R.val[p] = P.val[j];
        }
    return R;
}

// helper::sparse::cscSpMM (helper_sparse.hpp:257-285) with the left and right
// operands given as compressed columns: column i of the result accumulates
// alpha_k * left[:, r_k] over the entries (r_k, alpha_k) of right[:, i] in
// order; each entry is updated as y + alpha*x, and an entry that becomes exactly
// zero is removed (and restarts from alpha*x if hit again, which is the same as
// adding to 0.0).  A dense accumulator gives the same values; the touched rows
// are emitted in increasing order, as the merge-based original does.
static void csc_columns(const std::vector<int> &lp, const std::vector<int> &li, const std::vector<double> &lv,
                        int L, const std::vector<int> &rp, const std::vector<int> &ri, const std::vector<double> &rv,
                        int c0, int c1, std::vector<int> &cnt, std::vector<int> &oi, std::vector<double> &ov) {
    std::vector<double> acc(L, 0.0);
    std::vector<int> stamp(L, -1);
    std::vector<int> touched;
    for (int c = c0; c < c1; c++) {
        touched.clear();
        for (int k = rp[c]; k < rp[c + 1]; k++) {
            const int src = ri[k];
            const double alpha = rv[k];
            for (int t = lp[src]; t < lp[src + 1]; t++) {
                const int row = li[t];
                if (stamp[row] != c) {
                    stamp[row] = c;
                    acc[row] = 0.0;
                    touched.push_back(row);
                }
                acc[row] = acc[row] + alpha * lv[t];
            }
        }
        std::sort(touched.begin(), touched.end());
        int k = 0;
        for (int row : touched) {
            if (std::fabs(acc[row]) == 0.0) continue;
            oi.push_back(row);
            ov.push_back(acc[row]);
            k++;
        }
        cnt[c] = k;
    }
}

// Columns are independent: blocks of columns run on host threads, each with
// its own accumulator, and are concatenated in order (the values and their
// order do not depend on the number of threads).
static void csc_product(const std::vector<int> &lp, const std::vector<int> &li, const std::vector<double> &lv,
                        int L, const std::vector<int> &rp, const std::vector<int> &ri, const std::vector<double> &rv,
                        int R, std::vector<int> &op, std::vector<int> &oi, std::vector<double> &ov) {
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    const int T = R < 20000 || host_serial() ? 1 : std::min(hw, 16);
    std::vector<int> cnt(R, 0);
    std::vector<std::vector<int>> pi(T);
    std::vector<std::vector<double>> pv(T);
    std::vector<std::thread> pool;
    for (int t = 0; t < T; t++) {
        const int c0 = (int)((long long)R * t / T), c1 = (int)((long long)R * (t + 1) / T);
        if (t + 1 < T)
            pool.emplace_back([&, t, c0, c1] { csc_columns(lp, li, lv, L, rp, ri, rv, c0, c1, cnt, pi[t], pv[t]); });
        else
            csc_columns(lp, li, lv, L, rp, ri, rv, c0, c1, cnt, pi[t], pv[t]);
    }
    for (auto &th : pool) th.join();
    op.assign(R + 1, 0);
    for (int c = 0; c < R; c++) op[c + 1] = op[c] + cnt[c];
    oi.clear();
    ov.clear();
    oi.reserve(op[R]);
    ov.reserve(op[R]);
    for (int t = 0; t < T; t++) {
        oi.insert(oi.end(), pi[t].begin(), pi[t].end());
        ov.insert(ov.end(), pv[t].begin(), pv[t].end());
    }
}

// get_coarse_matrix (helper_multigrid.hpp:564-586): the reference passes CSR
// arrays where compressed columns are expected, so the first product forms
// T = A^T P and the second P^T T; read back as CSR this is C = P^T A P.
static CsrD galerkin(const CsrD &A, const CsrD &P, const CsrD &R) {
    std::vector<int> tp, ti, cp, ci;
    std::vector<double> tv, cv;
    csc_product(A.rptr, A.cind, A.val, A.n, R.rptr, R.cind, R.val, P.m, tp, ti, tv);
    csc_product(P.rptr, P.cind, P.val, P.m, tp, ti, tv, P.m, cp, ci, cv);
    CsrD C;
    C.n = C.m = P.m;
    C.rptr = std::move(cp);
    C.cind = std::move(ci);
    C.val = std::move(cv);
    return C;
}

void rs_level(const CsrD &A, double theta, CsrD &CA, CsrD &P, CsrD &R) {
    if (theta <= 0 || 1 < theta) throw SetupError{"Theta must be in 0 < theta <= 1"};
    CsrD S, W;
    strong_weak(A, theta, S, W);
    Pattern St = transpose_pattern(S);
    std::vector<int> is_coarse;
    rs_first_pass(S, St, is_coarse);
    rs_second_pass(S, is_coarse);
    P = interpolation(A, S, W, is_coarse);
    R = transpose(P);
    CA = galerkin(A, P, R);
}

RsChain rs_chain(const CsrD &A, double theta, int max_levels, int coarse_size) {
    RsChain ch;
    ch.CA.emplace_back();
    ch.P.emplace_back();
    ch.R.emplace_back();
    rs_level(A, theta, ch.CA[0], ch.P[0], ch.R[0]);
    int depth = 1;
    while (max_levels > depth && ch.CA[depth - 1].n > coarse_size) {
        // a coarsening step that barely shrinks the operator ends the chain
        // (only outside the reference's rule, coarse_size 2000)
        if (coarse_size != 2000 && depth >= 2 && ch.CA[depth - 1].n * 10 > ch.CA[depth - 2].n * 9) break;
        depth++;
        CsrD ca, p, r;
        rs_level(ch.CA[depth - 2], theta, ca, p, r);
        ch.CA.push_back(std::move(ca));
        ch.P.push_back(std::move(p));
        ch.R.push_back(std::move(r));
    }
    return ch;
}

// ============================================================= smoother splits

void sor_split(const CsrD &A, double omega, CsrD &LD, CsrD &U) {
    const int N = A.n;
    LD.n = LD.m = U.n = U.m = N;
    LD.rptr.assign(N + 1, 0);
    U.rptr.assign(N + 1, 0);
    LD.cind.clear(); LD.val.clear(); U.cind.clear(); U.val.clear();
    for (int i = 0; i < N; i++) {
        // split "LD-U" (helper_matrix.hpp:530-604): cind <= i to LD in row order
        int last_ld = -1;
        for (int j = A.rptr[i]; j < A.rptr[i + 1]; j++)
            if (A.cind[j] <= i) {
                LD.cind.push_back(A.cind[j]);
                LD.val.push_back(A.val[j]);
                last_ld = (int)LD.val.size() - 1;
            }
        // the last LD entry of the row is taken as the diagonal
        // (stationary.hpp:209-217): U gets (1 - 1/omega) d first, LD keeps d / omega
        const double d = last_ld >= 0 ? LD.val[last_ld] : 0.0;
        const int dcol = last_ld >= 0 ? LD.cind[last_ld] : 0;
        U.cind.push_back(dcol);
        U.val.push_back((1 - 1.0 / omega) * d);
        if (last_ld >= 0) LD.val[last_ld] = 1.0 / omega * d;
        for (int j = A.rptr[i]; j < A.rptr[i + 1]; j++)
            if (A.cind[j] > i) {
                U.cind.push_back(A.cind[j]);
                U.val.push_back(A.val[j]);
            }
        LD.rptr[i + 1] = (int)LD.cind.size();
        U.rptr[i + 1] = (int)U.cind.size();
    }
}

void block_sor_split(const CsrD &A, double omega, int nb, CsrD &LD, CsrD &U, std::vector<int> &bj) {
    const int N = A.n;
    const int size = (N + nb - 1) / nb;
    bj.assign(nb + 1, 0);
    for (int b = 0; b < nb; b++) bj[b + 1] = bj[b] + size;
    bj[nb] = N;
    LD.n = LD.m = U.n = U.m = N;
    LD.rptr.assign(N + 1, 0);
    U.rptr.assign(N + 1, 0);
    LD.cind.clear(); LD.val.clear(); U.cind.clear(); U.val.clear();
    for (int i = 0; i < N; i++) {
        const int left = bj[i / size];
        for (int j = A.rptr[i]; j < A.rptr[i + 1]; j++) {
            const int c = A.cind[j];
            if (c == i) {
                LD.cind.push_back(c); LD.val.push_back((1.0 / omega) * A.val[j]);
                U.cind.push_back(c); U.val.push_back((1 - 1.0 / omega) * A.val[j]);
            } else if (left <= c && c < i) {
                LD.cind.push_back(c); LD.val.push_back(A.val[j]);
            } else {
                U.cind.push_back(c); U.val.push_back(A.val[j]);
            }
        }
        LD.rptr[i + 1] = (int)LD.cind.size();
        U.rptr[i + 1] = (int)U.cind.size();
    }
}

static CsrD filter_rows(const CsrD &A, int mode) {  // 0: LDinv, 1: L, 2: DinvU
    CsrD B;
    B.n = A.n;
    B.m = A.m;
    B.rptr.assign(A.n + 1, 0);
    for (int i = 0; i < A.n; i++) {
        for (int j = A.rptr[i]; j < A.rptr[i + 1]; j++) {
            const int c = A.cind[j];
            if (c == i && mode != 1) {
                B.cind.push_back(c); B.val.push_back(1 / A.val[j]);
            } else if ((mode == 0 || mode == 1) && c < i) {
                B.cind.push_back(c); B.val.push_back(A.val[j]);
            } else if (mode == 2 && c > i) {
                B.cind.push_back(c); B.val.push_back(A.val[j]);
            }
        }
        B.rptr[i + 1] = (int)B.cind.size();
    }
    return B;
}
CsrD extract_ldinv(const CsrD &A) { return filter_rows(A, 0); }
CsrD extract_l(const CsrD &A) { return filter_rows(A, 1); }
CsrD extract_dinvu(const CsrD &A) { return filter_rows(A, 2); }

// helper::matrix::ilu (helper_matrix.hpp:978-1061), row by row with a dense
// work row: columns are eliminated in increasing order; an existing entry
// becomes a - pivot*u, a fill-in entry (-pivot)*u; no entry is dropped.  A row
// without a stored diagonal keeps the previous pivot, as the original does.
CsrD ilu_full(const CsrD &A) {
    const int N = A.n;
    CsrD F;
    F.n = F.m = N;
    F.rptr.assign(N + 1, 0);
    if (N == 0) return F;
    std::vector<double> w(N, 0.0);
    std::vector<char> nz(N, 0);
    std::vector<int> diagpos(N, -1);
    for (int j = A.rptr[0]; j < A.rptr[1]; j++) {
        F.cind.push_back(A.cind[j]);
        F.val.push_back(A.val[j]);
        if (A.cind[j] == 0) diagpos[0] = j - A.rptr[0];
    }
    F.rptr[1] = (int)F.cind.size();
    double pivot = 0;
    for (int i = 1; i < N; i++) {
        int lo = N;
        for (int j = A.rptr[i]; j < A.rptr[i + 1]; j++) {
            const int c = A.cind[j];
            w[c] = A.val[j];
            nz[c] = 1;
            lo = std::min(lo, c);
        }
        for (int k = lo; k < i; k++) {
            if (!nz[k]) continue;
            const int rs = F.rptr[k], re = F.rptr[k + 1];
            int dj = diagpos[k] >= 0 ? rs + diagpos[k] : -1;
            if (dj >= 0) pivot = w[k] / F.val[dj];
            w[k] = pivot;
            if (dj < 0) continue;
            for (int t = dj + 1; t < re; t++) {
                const int c = F.cind[t];
                if (nz[c]) {
                    w[c] = w[c] - pivot * F.val[t];
                } else {
                    nz[c] = 1;
                    w[c] = -pivot * F.val[t];
                }
            }
        }
        const int base = (int)F.cind.size();
        for (int c = lo; c < N; c++) {
            if (!nz[c]) continue;
            if (c == i) diagpos[i] = (int)F.cind.size() - base;
            F.cind.push_back(c);
            F.val.push_back(w[c]);
            nz[c] = 0;
            w[c] = 0.0;
        }
        F.rptr[i + 1] = (int)F.cind.size();
    }
    return F;
}

// ================================================================ quantisation

static CsrI shell_of(const CsrD &A) {
    CsrI B;
    B.n = A.n;
    B.m = A.m;
    B.rptr = A.rptr;
    B.cind = A.cind;
    B.val.resize(A.val.size());
    return B;
}

CsrI to_fixed(const CsrD &A, int bit) {
    CsrI B = shell_of(A);
    const double fact = (double)(1 << bit);
    for (size_t j = 0; j < A.val.size(); j++) B.val[j] = cvtt_i32(A.val[j] * fact);
    B.bit = bit;
    return B;
}

CsrI to_flex(const CsrD &A) {
    double mx = 0;
    for (double v : A.val)
        if (std::fabs(v) > mx) mx = std::fabs(v);
    CsrI B = shell_of(A);
    B.bit = flex_bit(mx);
    for (size_t j = 0; j < A.val.size(); j++) B.val[j] = quantize(A.val[j], B.bit);
    return B;
}

static void diag_offdiag_max(const CsrD &A, double &mx, double &dmx) {
    mx = 0;
    dmx = 0;
    for (int i = 0; i < A.n; i++)
        for (int j = A.rptr[i]; j < A.rptr[i + 1]; j++) {
            const double a = std::fabs(A.val[j]);
            if (A.cind[j] == i) {
                if (a > dmx) dmx = a;
            } else if (a > mx) {
                mx = a;
            }
        }
}

static CsrI quantize_split(const CsrD &A, int bit, int dbit) {
    CsrI B = shell_of(A);
    B.bit = bit;
    B.dbit = dbit;
    for (int i = 0; i < A.n; i++)
        for (int j = A.rptr[i]; j < A.rptr[i + 1]; j++)
            B.val[j] = quantize(A.val[j], A.cind[j] == i ? dbit : bit);
    return B;
}

CsrI to_ldtri_flex(const CsrD &LDinv) {
    double mx, dmx;
    diag_offdiag_max(LDinv, mx, dmx);
    return quantize_split(LDinv, flex_bit(mx), flex_bit(dmx));
}

CsrI to_ltri_flex(const CsrD &L) {
    double mx = 0;
    for (double v : L.val)
        if (std::fabs(v) > mx) mx = std::fabs(v);
    CsrI B = shell_of(L);
    B.bit = while_bit(mx);
    for (size_t j = 0; j < L.val.size(); j++) B.val[j] = quantize(L.val[j], B.bit);
    return B;
}

CsrI to_dutri_flex(const CsrD &DinvU) {
    double mx, dmx;
    diag_offdiag_max(DinvU, mx, dmx);
    return quantize_split(DinvU, while_bit(mx), while_bit(dmx));
}

// ================================================================= hierarchies

std::vector<int> greedy_colouring(const CsrD &A, int *ncolors, int max_colours) {
    const int N = A.n;
    // symmetrised adjacency without the diagonal
    std::vector<int> deg(N, 0);
    for (int i = 0; i < N; i++)
        for (int j = A.rptr[i]; j < A.rptr[i + 1]; j++)
            if (A.cind[j] != i) {
                deg[i]++;
                deg[A.cind[j]]++;
            }
    std::vector<int> ap(N + 1, 0);
    for (int i = 0; i < N; i++) ap[i + 1] = ap[i] + deg[i];
    std::vector<int> adj(ap[N]), fill(ap.begin(), ap.end() - 1);
    for (int i = 0; i < N; i++)
        for (int j = A.rptr[i]; j < A.rptr[i + 1]; j++) {
            const int c = A.cind[j];
            if (c == i) continue;
            adj[fill[i]++] = c;
            adj[fill[c]++] = i;
        }
    // colour k: sweep the rows in order, take every uncoloured row that has no
    // neighbour of colour k yet
    std::vector<int> col(N, -1);
    int k = 0, left = N;
    while (left > 0 && (max_colours <= 0 || k < max_colours)) {
        for (int i = 0; i < N; i++) {
            if (col[i] >= 0) continue;
            bool adjacent = false;
            for (int t = ap[i]; t < ap[i + 1]; t++)
                if (col[adj[t]] == k) {
                    adjacent = true;
                    break;
                }
            if (adjacent) continue;
            col[i] = k;
            left--;
        }
        k++;
    }
    if (left > 0) {
        // capped: every remaining row takes the colour with the fewest coloured
        // neighbours (lowest colour on ties); its same-colour couplings then act
        // through U, i.e. Jacobi-like within the colour
        std::vector<int> cnt(k, 0);
        for (int i = 0; i < N; i++) {
            if (col[i] >= 0) continue;
            std::fill(cnt.begin(), cnt.end(), 0);
            for (int t = ap[i]; t < ap[i + 1]; t++)
                if (col[adj[t]] >= 0) cnt[col[adj[t]]]++;
            col[i] = (int)(std::min_element(cnt.begin(), cnt.end()) - cnt.begin());
        }
    }
    if (ncolors) *ncolors = k;
    return col;
}

void mc_sor_split(const CsrD &A, double omega, const std::vector<int> &col, CsrD &LD, CsrD &U) {
    const int N = A.n;
    LD.n = LD.m = U.n = U.m = N;
    LD.rptr.assign(N + 1, 0);
    U.rptr.assign(N + 1, 0);
    LD.cind.clear(); LD.val.clear(); U.cind.clear(); U.val.clear();
    for (int i = 0; i < N; i++) {
        double d = 0;
        for (int j = A.rptr[i]; j < A.rptr[i + 1]; j++) {
            const int c = A.cind[j];
            if (c == i) {
                d = A.val[j];
            } else if (col[c] < col[i]) {
                LD.cind.push_back(c);
                LD.val.push_back(A.val[j]);
            }
        }
        LD.cind.push_back(i);
        LD.val.push_back(1.0 / omega * d);
        U.cind.push_back(i);
        U.val.push_back((1 - 1.0 / omega) * d);
        for (int j = A.rptr[i]; j < A.rptr[i + 1]; j++) {
            const int c = A.cind[j];
            if (c != i && col[c] >= col[i]) {
                U.cind.push_back(c);
                U.val.push_back(A.val[j]);
            }
        }
        LD.rptr[i + 1] = (int)LD.cind.size();
        U.rptr[i + 1] = (int)U.cind.size();
    }
}

void jacobi_sor_split(const CsrD &A, double omega, CsrD &LD, CsrD &U, std::vector<int> &colour) {
    const int N = A.n;
    LD.n = LD.m = U.n = U.m = N;
    LD.rptr.assign(N + 1, 0);
    U.rptr.assign(N + 1, 0);
    LD.cind.clear(); LD.val.clear(); U.cind.clear(); U.val.clear();
    colour.resize(N);
    for (int i = 0; i < N; i++) {
        colour[i] = i / kJacobiSorChunk;
        const int left = colour[i] * kJacobiSorChunk;  // the first row of row i's chunk
        for (int j = A.rptr[i]; j < A.rptr[i + 1]; j++) {
            const int c = A.cind[j];
            const double v = A.val[j];
            if (c == i) {
                LD.cind.push_back(c);
                LD.val.push_back(1.0 / omega * v);
                U.cind.push_back(c);
                U.val.push_back((1 - 1.0 / omega) * v);
            } else if (c < left) {
                LD.cind.push_back(c);
                LD.val.push_back(v);
            } else {
                U.cind.push_back(c);
                U.val.push_back(v);
            }
        }
        LD.rptr[i + 1] = (int)LD.cind.size();
        U.rptr[i + 1] = (int)U.cind.size();
    }
}

// LD with its diagonal (the last entry of each row) inverted: extractLDinv for a
// split whose couplings may lie on either side of the diagonal (colour order).
static CsrD invert_last(const CsrD &LD) {
    CsrD B = LD;
    for (int i = 0; i < B.n; i++)
        if (B.rptr[i + 1] > B.rptr[i]) B.val[B.rptr[i + 1] - 1] = 1 / B.val[B.rptr[i + 1] - 1];
    return B;
}

static void smoother_split(const CsrD &A, const SmootherSpec &sm, int level, CsrD &LD, CsrD &U,
                           std::vector<int> &bj, std::vector<int> &colour) {
    colour.clear();
    bj.clear();
    if (sm.multicolor == 2) {
        jacobi_sor_split(A, sm.omega, LD, U, colour);
    } else if (sm.multicolor) {
        int nc = 0;
        colour = greedy_colouring(A, &nc, sm.cap(level));
        mc_sor_split(A, sm.omega, colour, LD, U);
    } else if (sm.block > 0) {
        block_sor_split(A, sm.omega, sm.block, LD, U, bj);
    } else {
        sor_split(A, sm.omega, LD, U);
    }
}

IntHierarchy build_int_hierarchy(const CsrD &A, const RsChain &chain, const SmootherSpec &sm) {
    IntHierarchy h;
    const int D = chain.depth();
    h.depth = D;
    h.smooth_iter = sm.iter;
    h.A0 = to_fixed(A, 30);
    // row scaling of the coarse operators and restrictions (INTAMG.hpp:165-211)
    std::vector<CsrD> CA = chain.CA, It = chain.R;
    std::vector<double> prev(A.n, 0.0), mx;
    auto scale_level = [&](int t, bool use_prev) {
        CsrD &C = CA[t];
        CsrD &R = It[t];
        mx.assign(C.n, 0.0);
        for (int i = 0; i < C.n; i++) {
            for (int j = C.rptr[i]; j < C.rptr[i + 1]; j++)
                if (std::abs(C.val[j]) > mx[i]) mx[i] = std::abs(C.val[j]);
            for (int j = C.rptr[i]; j < C.rptr[i + 1]; j++) C.val[j] /= mx[i];
            for (int j = R.rptr[i]; j < R.rptr[i + 1]; j++) R.val[j] /= mx[i];
            if (!use_prev) continue;
            for (int j = R.rptr[i]; j < R.rptr[i + 1]; j++) R.val[j] *= prev[R.cind[j]];
        }
    };
    for (int d = 2; d <= D; d++) {
        scale_level(d - 2, d != 2);
        std::copy(mx.begin(), mx.end(), prev.begin());
    }
    // the coarsest level always multiplies by prev; with a single coarse level
    // prev is still all zero, so the restriction becomes zero (INTAMG.hpp:197-211)
    scale_level(D - 1, true);

    // the levels' smoother splits and conversions are independent: host threads
    h.LD.resize(D);
    h.U.resize(D);
    h.bj.resize(D);
    h.colour.resize(D);
    h.CA.resize(D - 1);
    h.P.resize(D);
    h.R.resize(D);
    parallel_tasks(2 * D + 1, [&](int t) {
        if (t < D) {
            const int l = t;
            const CsrD &Al = l == 0 ? A : CA[l - 1];
            CsrD LD, U;
            smoother_split(Al, sm, l, LD, U, h.bj[l], h.colour[l]);
            h.LD[l] = to_ldtri_flex(sm.multicolor ? invert_last(LD) : extract_ldinv(LD));
            h.U[l] = to_flex(U);
        } else if (t < 2 * D) {
            const int i = t - D;
            if (i < D - 1) h.CA[i] = to_flex(CA[i]);
            h.P[i] = to_flex(chain.P[i]);
            h.R[i] = to_flex(It[i]);
        } else {
            CsrD F = ilu_full(CA[D - 1]);
            h.LUL = to_ltri_flex(extract_l(F));
            h.LUU = to_dutri_flex(extract_dinvu(F));
        }
    });
    return h;
}

template <typename T>
static CsrT<T> convert(const CsrD &A) {
    CsrT<T> B;
    B.n = A.n;
    B.m = A.m;
    B.rptr = A.rptr;
    B.cind = A.cind;
    B.val.resize(A.val.size());
    for (size_t j = 0; j < A.val.size(); j++) B.val[j] = (T)A.val[j];
    return B;
}

template <typename T>
static FpHierarchy<T> build_fp(const CsrD &A, const RsChain &chain, const SmootherSpec &sm) {
    FpHierarchy<T> h;
    const int D = chain.depth();
    h.depth = D;
    h.smooth_iter = sm.iter;
    h.A0 = convert<T>(A);
    h.LD.resize(D);
    h.U.resize(D);
    h.bj.resize(D);
    h.colour.resize(D);
    h.CA.resize(D - 1);
    h.P.resize(D);
    h.R.resize(D);
    parallel_tasks(2 * D + 1, [&](int t) {
        if (t < D) {
            const int l = t;
            const CsrD &Al = l == 0 ? A : chain.CA[l - 1];
            CsrD LD, U;
            smoother_split(Al, sm, l, LD, U, h.bj[l], h.colour[l]);
            h.LD[l] = convert<T>(sm.multicolor ? invert_last(LD) : extract_ldinv(LD));
            h.U[l] = convert<T>(U);
        } else if (t < 2 * D) {
            const int i = t - D;
            if (i < D - 1) h.CA[i] = convert<T>(chain.CA[i]);
            h.P[i] = convert<T>(chain.P[i]);
            h.R[i] = convert<T>(chain.R[i]);
        } else {
            CsrD F = ilu_full(chain.CA[D - 1]);
            h.LUL = convert<T>(extract_l(F));
            h.LUU = convert<T>(extract_dinvu(F));
        }
    });
    return h;
}

FpHierarchy<double> build_f64_hierarchy(const CsrD &A, const RsChain &chain, const SmootherSpec &sm) {
    return build_fp<double>(A, chain, sm);
}
FpHierarchy<float> build_f32_hierarchy(const CsrD &A, const RsChain &chain, const SmootherSpec &sm) {
    return build_fp<float>(A, chain, sm);
}

}  // namespace sagb
