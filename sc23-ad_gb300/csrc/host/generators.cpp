#include "generators.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "sort.hpp"

namespace sagb {

uint64_t splitmix64_at(uint64_t seed, uint64_t i) {
    uint64_t z = seed + i * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

double uniform01_at(uint64_t seed, uint64_t i) {
    return (double)(splitmix64_at(seed, i) >> 11) * (1.0 / 9007199254740992.0);
}

// Assemble a structured-grid operator: for each row, the neighbours at the
// given offsets (sorted by the resulting column), values from coef(row, k).
template <typename F>
static CsrD structured(const int *dims, int nd, const int (*offs)[3], int noff, F coef) {
    int64_t N = 1;
    for (int a = 0; a < nd; a++) N *= dims[a];
    int64_t stride[3] = {1, dims[0], nd > 1 ? (int64_t)dims[0] * dims[1] : 1};
    // sort offsets by column displacement so that rows come out sorted
    int order[27];
    for (int k = 0; k < noff; k++) order[k] = k;
    auto disp = [&](int k) {
        int64_t d = 0;
        for (int a = 0; a < nd; a++) d += offs[k][a] * stride[a];
        return d;
    };
    for (int a = 1; a < noff; a++)
        for (int b = a; b > 0 && disp(order[b]) < disp(order[b - 1]); b--) std::swap(order[b], order[b - 1]);
    CsrD A;
    A.n = A.m = (int)N;
    A.rptr.assign(N + 1, 0);
    A.cind.reserve(N * noff);
    A.val.reserve(N * noff);
    int c[3] = {0, 0, 0};
    for (int64_t row = 0; row < N; row++) {
        int64_t t = row;
        for (int a = 0; a < nd; a++) {
            c[a] = (int)(t % dims[a]);
            t /= dims[a];
        }
        for (int q = 0; q < noff; q++) {
            const int k = order[q];
            bool ok = true;
            for (int a = 0; a < nd; a++) {
                const int v = c[a] + offs[k][a];
                ok &= v >= 0 && v < dims[a];
            }
            if (!ok) continue;
            A.cind.push_back((int)(row + disp(k)));
            A.val.push_back(coef(row, k));
        }
        A.rptr[row + 1] = (int)A.cind.size();
    }
    return A;
}

static const int kOff2d5[5][3] = {{0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}};
static const int kOff3d7[7][3] = {{0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};

CsrD gen_poisson2d(int n) {
    int d[2] = {n, n};
    return structured(d, 2, kOff2d5, 5, [](int64_t, int k) { return k == 0 ? 4.0 : -1.0; });
}

CsrD gen_poisson3d(int n) {
    int d[3] = {n, n, n};
    return structured(d, 3, kOff3d7, 7, [](int64_t, int k) { return k == 0 ? 6.0 : -1.0; });
}

CsrD gen_aniso2d(int n, double eps) {
    int d[2] = {n, n};
    return structured(d, 2, kOff2d5, 5, [eps](int64_t, int k) {
        if (k == 0) return 2.0 + 2.0 * eps;
        return k <= 2 ? -1.0 : -eps;
    });
}

CsrD gen_stencil27(int n, uint64_t seed) {
    int offs[27][3];
    int q = 0;
    for (int c = -1; c <= 1; c++)
        for (int b = -1; b <= 1; b++)
            for (int a = -1; a <= 1; a++) {
                offs[q][0] = a;
                offs[q][1] = b;
                offs[q][2] = c;
                q++;
            }
    int d[3] = {n, n, n};
    return structured(d, 3, offs, 27, [seed](int64_t row, int k) {
        if (k == 13) return 26.0 + (0.1 + 0.9 * uniform01_at(seed, (uint64_t)row + 1));
        return -1.0;
    });
}

CsrD gen_convdiff3d(int n, double pe) {
    const double h = 1.0 / (n + 1);
    const double b = pe / std::sqrt(3.0);
    const double diag = 6.0 + 3.0 * h * b;
    const double up = -1.0 - h * b;
    int d[3] = {n, n, n};
    return structured(d, 3, kOff3d7, 7, [=](int64_t, int k) {
        if (k == 0) return diag;
        return (k % 2 == 0) ? up : -1.0;  // offsets 2, 4, 6 are the minus side
    });
}

CsrD gen_varcoef3d(int n, double sigma, uint64_t seed) {
    const int64_t N = (int64_t)n * n * n;
    std::vector<double> k(N);
    const double two_pi = 2.0 * M_PI;
    for (int64_t i = 0; i < N; i++) {
        const double u1 = uniform01_at(seed, (uint64_t)i + 1);
        const double u2 = uniform01_at(seed + 1, (uint64_t)i + 1);
        const double z = std::sqrt(-2.0 * std::log(1.0 - u1)) * std::cos(two_pi * u2);
        k[i] = std::exp(sigma * z);
    }
    const int64_t stride[3] = {1, n, (int64_t)n * n};
    CsrD A;
    A.n = A.m = (int)N;
    A.rptr.assign(N + 1, 0);
    for (int64_t row = 0; row < N; row++) {
        const int c[3] = {(int)(row % n), (int)((row / n) % n), (int)(row / ((int64_t)n * n))};
        // face coefficients in the order +x, -x, +y, -y, +z, -z
        double kf[6];
        bool in[6];
        double diag = 0;
        for (int ax = 0; ax < 3; ax++)
            for (int sgn = 0; sgn < 2; sgn++) {
                const int f = 2 * ax + sgn;
                const int v = c[ax] + (sgn == 0 ? 1 : -1);
                in[f] = v >= 0 && v < n;
                if (in[f]) {
                    const double kn = k[row + (sgn == 0 ? 1 : -1) * stride[ax]];
                    kf[f] = 2.0 * k[row] * kn / (k[row] + kn);
                } else {
                    kf[f] = k[row];
                }
                diag += kf[f];
            }
        // emit in column order: -z, -y, -x, diag, +x, +y, +z
        const int ord[7] = {5, 3, 1, -1, 0, 2, 4};
        for (int q = 0; q < 7; q++) {
            const int f = ord[q];
            if (f < 0) {
                A.cind.push_back((int)row);
                A.val.push_back(diag);
            } else if (in[f]) {
                const int ax = f / 2;
                A.cind.push_back((int)(row + (f % 2 == 0 ? 1 : -1) * stride[ax]));
                A.val.push_back(-kf[f]);
            }
        }
        A.rptr[row + 1] = (int)A.cind.size();
    }
    return A;
}

void gen_rhs(const CsrD &A, uint64_t seed, double *xstar, double *b) {
    for (int i = 0; i < A.n; i++) xstar[i] = uniform01_at(seed, (uint64_t)i + 1) * 2.0 - 1.0;
    for (int i = 0; i < A.n; i++) {
        double s = 0.0;
        for (int j = A.rptr[i]; j < A.rptr[i + 1]; j++) s += A.val[j] * xstar[A.cind[j]];
        b[i] = s;
    }
}

// ------------------------------------------------------------ Matrix Market

CsrD read_matrix_market(const char *path) {
    FILE *f = fopen(path, "rb");
    if (!f) throw SetupError{std::string("cannot open ") + path};
    std::string data;
    {
        char buf[1 << 16];
        size_t k;
        while ((k = fread(buf, 1, sizeof buf, f)) > 0) data.append(buf, k);
        fclose(f);
    }
    if (data.empty()) throw SetupError{"empty Matrix Market file"};
    const char *p = data.c_str();
    const char *hdr = "%%MatrixMarket matrix coordinate";
    if (strncmp(p, hdr, strlen(hdr)) != 0) throw SetupError{"invalid Matrix Market header"};
    p += strlen(hdr);
    char type[64] = {0}, shape[64] = {0};
    if (sscanf(p, "%63s %63s", type, shape) != 2) throw SetupError{"invalid Matrix Market header"};
    if (strcmp(type, "real") != 0 && strcmp(type, "integer") != 0) throw SetupError{std::string(type) + " is not supported"};
    const bool sym = strcmp(shape, "symmetric") == 0;
    if (!sym && strcmp(shape, "general") != 0) throw SetupError{std::string(shape) + " is not supported"};
    while (*p && *p != '\n') p++;
    if (*p) p++;
    while (*p == '%') {
        while (*p && *p != '\n') p++;
        if (*p) p++;
    }
    char *end;
    const long N = strtol(p, &end, 10);
    const long M = strtol(end, &end, 10);
    const long PE = strtol(end, &end, 10);
    p = end;
    if (N <= 0 || M <= 0 || PE < 0) throw SetupError{"invalid Matrix Market size line"};
    std::vector<int> row, col;
    std::vector<double> val;
    row.reserve(PE);
    col.reserve(PE);
    val.reserve(PE);
    for (long e = 0; e < PE; e++) {
        const long r = strtol(p, &end, 10);
        const long c = strtol(end, &end, 10);
        const double v = strtod(end, &end);
        if (end == p) throw SetupError{"truncated Matrix Market file"};
        p = end;
        if (v == 0) continue;  // has_zeros == false
        row.push_back((int)r - 1);
        col.push_back((int)c - 1);
        val.push_back(v);
    }
    const int nnz = (int)row.size();
    if (nnz > 0) hoare_sort(0, nnz - 1, true, row.data(), col.data(), val.data());
    CsrD A;
    A.n = (int)N;
    A.m = (int)M;
    A.rptr.assign(N + 1, 0);
    int cnt = 0;
    for (int i = 0; i < N; i++) {
        int num = 0;
        while (cnt < nnz && row[cnt] == i) { num++; cnt++; }
        A.rptr[i + 1] = A.rptr[i] + num;
        if (num > 1) hoare_sort(A.rptr[i], A.rptr[i + 1] - 1, true, col.data(), val.data());
    }
    A.cind.assign(col.begin(), col.begin() + nnz);
    A.val.assign(val.begin(), val.begin() + nnz);
    if (sym) {
        // helper::matrix::expand(..., "L") (helper_matrix.hpp:730-766): the stored
        // lower triangle plus its transpose without the diagonal
        CsrD T;
        T.n = (int)M;
        T.rptr.assign(M + 1, 0);
        for (int c : A.cind) T.rptr[c + 1]++;
        for (long i = 0; i < M; i++) T.rptr[i + 1] += T.rptr[i];
        T.cind.resize(nnz);
        T.val.resize(nnz);
        std::vector<int> fill(T.rptr.begin(), T.rptr.end() - 1);
        for (int i = 0; i < A.n; i++)
            for (int j = A.rptr[i]; j < A.rptr[i + 1]; j++) {
                const int q = fill[A.cind[j]]++;
                T.cind[q] = i;
                T.val[q] = A.val[j];
            }
        CsrD E;
        E.n = A.n;
        E.m = A.m;
        E.rptr.assign(A.n + 1, 0);
        for (int i = 0; i < A.n; i++) {
            for (int j = A.rptr[i]; j < A.rptr[i + 1]; j++) {
                E.cind.push_back(A.cind[j]);
                E.val.push_back(A.val[j]);
            }
            for (int j = T.rptr[i] + 1; j < T.rptr[i + 1]; j++) {
                E.cind.push_back(T.cind[j]);
                E.val.push_back(T.val[j]);
            }
            E.rptr[i + 1] = (int)E.cind.size();
        }
        return E;
    }
    return A;
}

}  // namespace sagb
