#include "features.hpp"

#include <algorithm>
#include <cmath>

namespace sagb {

static double lg2(double x) { return std::log2(std::max(x, 1e-300)); }

// value of entry (i, j) of a row-sorted CSR, 0 when absent
static double entry(const CsrD &A, int i, int j) {
    const int *b = A.cind.data() + A.rptr[i], *e = A.cind.data() + A.rptr[i + 1];
    const int *p = std::lower_bound(b, e, j);
    if (p != e && *p == j) return A.val[p - A.cind.data()];
    for (const int *q = b; q != e; q++)  // rows that are not sorted
        if (*q == j) return A.val[q - A.cind.data()];
    return 0.0;
}

void bit_features(const CsrD &A, const IntHierarchy &h, double ratio, float *out) {
    const int N = A.n;
    const double nnz = (double)A.nnz();
    int maxrow = 0;
    double dd_sum = 0, dd_min = 1e30, asym = 0, absum = 0, npos = 0, noff = 0;
    for (int i = 0; i < N; i++) {
        maxrow = std::max(maxrow, A.rptr[i + 1] - A.rptr[i]);
        double d = 0, off = 0;
        for (int j = A.rptr[i]; j < A.rptr[i + 1]; j++) {
            const int c = A.cind[j];
            const double v = A.val[j];
            absum += std::fabs(v);
            if (c == i) {
                d = std::fabs(v);
                continue;
            }
            off += std::fabs(v);
            noff += 1;
            if (v > 0) npos += 1;
            if (c < N) asym += std::fabs(v - entry(A, c, i));
        }
        const double r = off > 0 ? std::min(d / off, 10.0) : 10.0;
        dd_sum += r;
        dd_min = std::min(dd_min, r);
    }
    double cplx = nnz;
    int bmin = 64, bmax = -64;
    double bsum = 0;
    int bcnt = 0;
    for (const CsrI &m : h.CA) {
        cplx += (double)m.nnz();
        bmin = std::min(bmin, m.bit);
        bmax = std::max(bmax, m.bit);
        bsum += m.bit;
        bcnt++;
    }
    int pr_min = 64;
    for (const CsrI &m : h.P) pr_min = std::min(pr_min, m.bit);
    for (const CsrI &m : h.R) pr_min = std::min(pr_min, m.bit);
    int ld_dmin = 64, ld_dmax = -64;
    for (const CsrI &m : h.LD) {
        ld_dmin = std::min(ld_dmin, m.dbit);
        ld_dmax = std::max(ld_dmax, m.dbit);
    }
    if (bcnt == 0) bmin = bmax = 0;
    if (pr_min == 64) pr_min = 0;
    if (ld_dmin == 64) ld_dmin = ld_dmax = 0;
    const int rule = rule_frac_bits(ratio, 1.0);
    const int coarse = h.LUL.n;
    float f[kNumFeatures] = {
        (float)lg2(N),
        (float)(N ? nnz / N : 0),
        (float)lg2(maxrow),
        (float)h.depth,
        (float)lg2(coarse > 0 ? coarse : 1),
        (float)(nnz > 0 ? cplx / nnz : 0),
        (float)std::min(std::max(lg2(ratio), -60.0), 60.0),
        (float)rule,
        (float)(N ? dd_sum / N : 0),
        (float)(N ? dd_min : 0),
        (float)(absum > 0 ? asym / absum : 0),
        (float)(noff > 0 ? npos / noff : 0),
        (float)bmin,
        (float)(bcnt ? bsum / bcnt : 0),
        (float)pr_min,
        (float)(h.LD.empty() ? 0 : h.LD[0].bit),
        (float)ld_dmin,
        (float)ld_dmax,
        (float)h.LUL.bit,
        (float)h.LUU.dbit,
    };
    std::copy(f, f + kNumFeatures, out);
}

}  // namespace sagb
