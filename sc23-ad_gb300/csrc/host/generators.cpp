#include "generators.hpp"

#include <sys/stat.h>

#include <algorithm>
#include <cctype>
#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <system_error>
#include <thread>

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

// ------------------------------------------------------- Matrix Market input
static std::vector<char> read_file(const char *path) {
    FILE *f = fopen(path, "rb");
    if (!f) throw SetupError{std::string("cannot open ") + path};
    std::vector<char> data;
    struct stat st;
    if (fstat(fileno(f), &st) == 0 && S_ISREG(st.st_mode) && st.st_size > 0) {
        data.resize((size_t)st.st_size);
        const size_t k = fread(data.data(), 1, data.size(), f);
        data.resize(k);
    } else {
        char buf[1 << 16];
        size_t k;
        while ((k = fread(buf, 1, sizeof buf, f)) > 0) data.insert(data.end(), buf, buf + k);
    }
    fclose(f);
    data.push_back('\0');
    return data;
}

static bool token_end(char ch) { return ch == '\0' || isspace((unsigned char)ch); }

// strtol / strtod on one token; the fast paths (plain decimal digits,
// std::from_chars, which rounds correctly like strtod) are taken only when
// they consume the whole whitespace-delimited token, otherwise the C library
// call decides
static long parse_long(const char *p, const char **end) {
    while (isspace((unsigned char)*p)) p++;
    const char *q = p;
    bool neg = false;
    if (*q == '-') {
        neg = true;
        q++;
    }
    if (*q >= '0' && *q <= '9') {
        long v = 0;
        int digits = 0;
        while (*q >= '0' && *q <= '9' && digits < 18) {
            v = v * 10 + (*q - '0');
            q++;
            digits++;
        }
        if (token_end(*q)) {
            *end = q;
            return neg ? -v : v;
        }
    }
    char *e;
    const long v = strtol(p, &e, 10);
    *end = e;
    return v;
}

static double parse_double(const char *p, const char *limit, const char **end) {
    while (isspace((unsigned char)*p)) p++;
    double v = 0;
    const auto r = std::from_chars(p, limit, v, std::chars_format::general);
    if (r.ec == std::errc() && r.ptr > p && token_end(*r.ptr)) {
        *end = r.ptr;
        return v;
    }
    char *e;
    v = strtod(p, &e);
    *end = e;
    return v;
}

struct MmPart {
    std::vector<int> row, col;
    std::vector<double> val;
    bool ok = true;
};

// the entries of [p, q), which starts and ends at line boundaries; a triple
// that does not end inside the range (a file that breaks entries across
// lines in a way the split does not see) marks the part as not ok
static void parse_part(const char *p, const char *q, const char *limit, MmPart &out) {
    while (true) {
        while (p < q && isspace((unsigned char)*p)) p++;
        if (p >= q) return;
        const char *e;
        const long r = parse_long(p, &e);
        if (e == p) break;
        const char *e2;
        const long c = parse_long(e, &e2);
        if (e2 == e) break;
        const char *e3;
        const double v = parse_double(e2, limit, &e3);
        if (e3 == e2 || e3 > q) break;
        out.row.push_back((int)r - 1);
        out.col.push_back((int)c - 1);
        out.val.push_back(v);
        p = e3;
    }
    out.ok = false;
}

CsrD read_matrix_market(const char *path) {
    const std::vector<char> buf = read_file(path);
    if (buf.size() <= 1) throw SetupError{"empty Matrix Market file"};
    const char *p = buf.data();
    const char *limit = buf.data() + buf.size() - 1;  // the terminating NUL
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
    // the entry lines in parts on host threads (line-aligned, kept in file order)
    const size_t len = (size_t)(limit - p);
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    const int T = (int)std::max<size_t>(1, std::min<size_t>((size_t)std::min(hw, 32), len >> 16));
    std::vector<const char *> cut(T + 1);
    cut[0] = p;
    cut[T] = limit;
    for (int t = 1; t < T; t++) {
        const char *c = std::max(cut[t - 1], p + len * t / T);
        while (c < limit && *c != '\n') c++;
        cut[t] = c < limit ? c + 1 : limit;
    }
    std::vector<MmPart> parts(T);
    {
        std::vector<std::thread> pool;
        for (int t = 1; t < T; t++) pool.emplace_back([&, t] { parse_part(cut[t], cut[t + 1], limit, parts[t]); });
        parse_part(cut[0], cut[1], limit, parts[0]);
        for (auto &th : pool) th.join();
    }
    // the first PE entries in file order; a part that stopped early ends the
    // entries there (what follows is not read, as in a sequential read)
    std::vector<int> row, col;
    std::vector<double> val;
    auto gather = [&](const std::vector<MmPart> &ps) {
        row.clear();
        col.clear();
        val.clear();
        long taken = 0;
        for (size_t t = 0; t < ps.size() && taken < PE; t++) {
            const MmPart &q = ps[t];
            for (size_t k = 0; k < q.row.size() && taken < PE; k++, taken++) {
                if (q.val[k] == 0) continue;  // has_zeros == false
                row.push_back(q.row[k]);
                col.push_back(q.col[k]);
                val.push_back(q.val[k]);
            }
            if (!q.ok) break;
        }
        return taken;
    };
    row.reserve(PE);
    col.reserve(PE);
    val.reserve(PE);
    long taken = gather(parts);
    if (taken < PE && T > 1) {
        // an entry broken across a split point: read the whole body in one part
        std::vector<MmPart> one(1);
        parse_part(p, limit, limit, one[0]);
        taken = gather(one);
    }
    if (taken < PE) throw SetupError{"truncated Matrix Market file"};
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
    col.resize(nnz);
    val.resize(nnz);
    A.cind = std::move(col);
    A.val = std::move(val);
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
        E.cind.reserve(2 * (size_t)nnz);
        E.val.reserve(2 * (size_t)nnz);
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

// ------------------------------------------------------------ binary CSR cache
// Our own format, in the host's byte order: the header, then rptr (int32,
// n + 1), cind (int32, nnz), val (float64, nnz).
namespace {
struct CsrFileHeader {
    char magic[8];
    int64_t n, m, nnz;
    int64_t src_size, src_mtime_ns;  // the Matrix Market file it came from (-1: none)
};
constexpr char kCsrMagic[8] = {'S', 'A', 'C', 'S', 'R', '0', '1', 0};

bool file_stamp(const char *path, int64_t *size, int64_t *mtime_ns) {
    struct stat st;
    if (stat(path, &st) != 0) return false;
    *size = (int64_t)st.st_size;
    *mtime_ns = (int64_t)st.st_mtim.tv_sec * 1000000000LL + (int64_t)st.st_mtim.tv_nsec;
    return true;
}
}  // namespace

void write_csr_binary(const CsrD &A, const char *path, int64_t src_size, int64_t src_mtime_ns) {
    const std::string tmp = std::string(path) + ".tmp";
    FILE *f = fopen(tmp.c_str(), "wb");
    if (!f) throw SetupError{std::string("cannot write ") + tmp};
    CsrFileHeader h;
    memcpy(h.magic, kCsrMagic, 8);
    h.n = A.n;
    h.m = A.m;
    h.nnz = A.nnz();
    h.src_size = src_size;
    h.src_mtime_ns = src_mtime_ns;
    bool ok = fwrite(&h, sizeof h, 1, f) == 1;
    ok = ok && fwrite(A.rptr.data(), sizeof(int), A.n + 1, f) == (size_t)A.n + 1;
    ok = ok && (h.nnz == 0 || fwrite(A.cind.data(), sizeof(int), h.nnz, f) == (size_t)h.nnz);
    ok = ok && (h.nnz == 0 || fwrite(A.val.data(), sizeof(double), h.nnz, f) == (size_t)h.nnz);
    ok = fclose(f) == 0 && ok;
    if (!ok || rename(tmp.c_str(), path) != 0) {
        remove(tmp.c_str());
        throw SetupError{std::string("cannot write ") + path};
    }
}

bool read_csr_binary(const char *path, CsrD &A, int64_t *src_size, int64_t *src_mtime_ns) {
    FILE *f = fopen(path, "rb");
    if (!f) return false;
    CsrFileHeader h;
    struct stat st;
    bool ok = fread(&h, sizeof h, 1, f) == 1 && memcmp(h.magic, kCsrMagic, 8) == 0 && h.n >= 0 && h.m >= 0 &&
              h.nnz >= 0 && h.n < INT32_MAX && h.m < INT32_MAX && h.nnz < INT32_MAX &&
              fstat(fileno(f), &st) == 0 &&
              (int64_t)st.st_size == (int64_t)sizeof h + 4 * (h.n + 1) + 12 * h.nnz;
    CsrD B;
    if (ok) {
        B.n = (int)h.n;
        B.m = (int)h.m;
        B.rptr.resize(h.n + 1);
        B.cind.resize(h.nnz);
        B.val.resize(h.nnz);
        ok = fread(B.rptr.data(), sizeof(int), h.n + 1, f) == (size_t)h.n + 1 &&
             (h.nnz == 0 || fread(B.cind.data(), sizeof(int), h.nnz, f) == (size_t)h.nnz) &&
             (h.nnz == 0 || fread(B.val.data(), sizeof(double), h.nnz, f) == (size_t)h.nnz);
    }
    fclose(f);
    if (!ok || B.rptr[0] != 0 || B.rptr[B.n] != h.nnz) return false;
    for (int i = 0; i < B.n; i++)
        if (B.rptr[i + 1] < B.rptr[i]) return false;
    for (int64_t j = 0; j < h.nnz; j++)
        if (B.cind[j] < 0 || B.cind[j] >= B.m) return false;
    A = std::move(B);
    if (src_size) *src_size = h.src_size;
    if (src_mtime_ns) *src_mtime_ns = h.src_mtime_ns;
    return true;
}

CsrD read_matrix_market_cached(const char *mm_path, const char *cache_path) {
    int64_t size = -1, mtime = -1;
    if (!file_stamp(mm_path, &size, &mtime)) throw SetupError{std::string("cannot open ") + mm_path};
    CsrD A;
    int64_t cs = 0, cm = 0;
    if (read_csr_binary(cache_path, A, &cs, &cm) && cs == size && cm == mtime) return A;
    A = read_matrix_market(mm_path);
    try {
        write_csr_binary(A, cache_path, size, mtime);
    } catch (const SetupError &) {
        // an unwritable cache only costs the next read its parse
    }
    return A;
}

}  // namespace sagb
