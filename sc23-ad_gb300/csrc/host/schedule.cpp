#include "schedule.hpp"

#include <algorithm>

namespace sagb {

TriSchedule build_tri_schedule(const int *rptr, const int *cind, int n, int kind, int rows_per_chunk,
                               int max_run_levels, const int *level_hint) {
    TriSchedule s;
    s.n = n;
    s.kind = kind;
    std::vector<int> level(n, 0);
    // dependencies: LD rows read columns < i (all but the last entry, D^-1);
    // L rows read every entry; DU rows read every entry but the first (D^-1)
    auto off_range = [&](int i, int &a, int &b) {
        a = rptr[i];
        b = rptr[i + 1];
        if (kind == TRI_LD) b = b - 1;
        if (kind == TRI_DU) a = a + 1;
        if (b < a) b = a;
    };
    int nlev = 0;
    if (level_hint) {
        for (int i = 0; i < n; i++) {
            int a, b;
            off_range(i, a, b);
            for (int j = a; j < b; j++)
                if (level_hint[cind[j]] >= level_hint[i]) throw SetupError{"level hint violates a dependency"};
            level[i] = level_hint[i];
            nlev = std::max(nlev, level[i] + 1);
        }
    } else if (kind == TRI_DU) {
        for (int i = n - 1; i >= 0; i--) {
            int a, b, lv = 0;
            off_range(i, a, b);
            for (int j = a; j < b; j++) lv = std::max(lv, level[cind[j]] + 1);
            level[i] = lv;
            nlev = std::max(nlev, lv + 1);
        }
    } else {
        for (int i = 0; i < n; i++) {
            int a, b, lv = 0;
            off_range(i, a, b);
            for (int j = a; j < b; j++) lv = std::max(lv, level[cind[j]] + 1);
            level[i] = lv;
            nlev = std::max(nlev, lv + 1);
        }
    }
    s.nlev = nlev;
    // counting sort by level, rows inside a level in increasing order (or
    // decreasing for the backward sweep, which keeps memory order monotone)
    std::vector<int> cnt(nlev + 1, 0);
    for (int i = 0; i < n; i++) cnt[level[i] + 1]++;
    for (int l = 0; l < nlev; l++) cnt[l + 1] += cnt[l];
    std::vector<int> lptr(cnt);
    s.lvl_ptr = lptr;
    s.perm.resize(n);
    if (kind == TRI_DU) {
        for (int i = n - 1; i >= 0; i--) s.perm[cnt[level[i]]++] = i;
    } else {
        for (int i = 0; i < n; i++) s.perm[cnt[level[i]]++] = i;
    }
    for (int l = 0; l < nlev; l++) s.max_level_rows = std::max(s.max_level_rows, lptr[l + 1] - lptr[l]);
    // off-diagonal entries in position order
    s.prp.assign(n + 1, 0);
    s.diag_src.assign(n, -1);
    for (int p = 0; p < n; p++) {
        int i = s.perm[p], a, b;
        off_range(i, a, b);
        s.prp[p + 1] = s.prp[p] + (b - a);
        if (kind == TRI_LD && rptr[i + 1] > rptr[i]) s.diag_src[p] = rptr[i + 1] - 1;
        if (kind == TRI_DU && rptr[i + 1] > rptr[i]) s.diag_src[p] = rptr[i];
    }
    s.pci.resize(s.prp[n]);
    s.src_idx.resize(s.prp[n]);
    for (int p = 0; p < n; p++) {
        int i = s.perm[p], a, b;
        off_range(i, a, b);
        for (int j = a; j < b; j++) {
            s.pci[s.prp[p] + (j - a)] = cind[j];
            s.src_idx[s.prp[p] + (j - a)] = j;
        }
    }
    // chunks: split big levels, merge runs of small ones
    s.sub_bound.clear();
    s.chunk_lv.clear();
    s.chunk_lv.push_back(0);
    int l = 0;
    while (l < nlev) {
        const int sz = lptr[l + 1] - lptr[l];
        if (sz > rows_per_chunk / 2) {
            // one or more chunks that each cover a slice of level l
            const int pieces = (sz + rows_per_chunk - 1) / rows_per_chunk;
            for (int q = 0; q < pieces; q++) {
                const int a = lptr[l] + (int)((int64_t)sz * q / pieces);
                s.sub_bound.push_back(a);
                s.sub_level.push_back(l);
                s.chunk_lv.push_back((int)s.sub_bound.size());
            }
            l++;
        } else {
            // a run of small levels in one chunk
            int rows = 0, runl = 0;
            while (l < nlev && runl < max_run_levels) {
                const int z = lptr[l + 1] - lptr[l];
                if (runl > 0 && (z > rows_per_chunk / 2 || rows + z > rows_per_chunk)) break;
                s.sub_bound.push_back(lptr[l]);
                s.sub_level.push_back(l);
                rows += z;
                runl++;
                l++;
            }
            s.chunk_lv.push_back((int)s.sub_bound.size());
        }
    }
    s.sub_bound.push_back(n);
    return s;
}

}  // namespace sagb
