// Reference harness: TEST INFRASTRUCTURE ONLY.
//
// Compiled (by oracle/Makefile) against the read-only reference Library headers of
// suzuki-hpc/SC23-AD.  It drives the reference's own public classes on a matrix
// read with the reference's own Matrix Market reader and dumps every array the
// solve phase touches, plus kernel input/output pairs, as raw little-endian files
// into an output directory.  tests/golden/make_golden.py packs those files into the
// committed fixtures.  Nothing in the product links or runs this file.
//
// Private members are reached with `#define private public` (for labelled
// sections) and with layout mirrors (for classes whose members are private by
// default).  The mirrors follow the member order of the reference classes:
//   CSR<Fixed<bit>>        matrix/spmat.hpp:56-61
//   CSRflex                matrix/spmat.hpp:89-94
//   ldtri::CSRflex         matrix/trimat/ldtri.hpp:120-125
//   ldtri::BJCSRflex       matrix/trimat/ldtri.hpp:462-468
//   ltri::CSRflex          matrix/trimat/ltri.hpp:88-93
//   dutri::CSRflex         matrix/trimat/dutri.hpp:98-103
//   direct::LUflex         solver/lu.hpp:71-74
//   CSR<T>                 matrix/spmat.hpp:21-26, ldtri::CSR<T> ldtri.hpp:19-24,
//   ltri::CSR<T> ltri.hpp:19-24, dutri::CSR<T> dutri.hpp:19-24, direct::LU<T> lu.hpp:11-14

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fcntl.h>
#include <iomanip>
#include <iostream>
#include <random>
#include <string>
#include <sys/mman.h>
#include <sys/stat.h>
#include <sys/time.h>
#include <type_traits>
#include <unistd.h>
#include <utility>
#include <vector>

#define private public
#include "timer.hpp"
#include "utils/utils.hpp"
#include "io/mm.hpp"
#include "matrix/spmat.hpp"
#include "matrix/trimat/spmat.hpp"
#include "blas/blas1.hpp"
#include "solver/gmres.hpp"
#include "solver/irsolver.hpp"
#include "preconditioner/INTAMG.hpp"
#include "smoother/stationary.hpp"
#undef private

using namespace senk;

// ---------------------------------------------------------------- layout mirrors
struct MFixed  { void *vp; int N, M; int *val, *cind, *rptr; };
struct MFlex   { void *vp; int N, M; int *val, *cind, *rptr; int bit; };
struct MLD     { void *vp; int N, M; int *val, *cind, *rptr; int bit, dbit; };
struct MBJ     { void *vp; int N, M; int *val, *cind, *rptr; int *bj_size, bj_num; int bit, dbit; };
struct MLT     { void *vp; int N, M; int *val, *cind, *rptr; int bit; };
struct MDU     { void *vp; int N, M; int *val, *cind, *rptr; int bit, dbit; };
struct MLUflex { void *L; void *U; int *temp; };
template <typename T> struct MCsrT { void *vp; int N, M; T *val; int *cind, *rptr; };
template <typename T> struct MLU { void *L; void *U; T *temp; };

static std::string g_out;

template <typename T>
static void dump(const std::string &name, const T *p, size_t n) {
    const char *suf = std::is_same_v<T, int> ? "i32" : std::is_same_v<T, long> ? "i64"
                    : std::is_same_v<T, double> ? "f64" : std::is_same_v<T, float> ? "f32" : "u8";
    std::string path = g_out + "/" + name + "." + suf;
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) { perror(path.c_str()); exit(2); }
    if (n) fwrite(p, sizeof(T), n, f);
    fclose(f);
}
static void dump_scalar_i(const std::string &name, long v) { dump(name, &v, 1); }

template <typename S>
static void dump_csr_int(const std::string &pfx, S *m, int bit, int dbit) {
    int N = m->N;
    dump(pfx + "_rptr", m->rptr, N + 1);
    dump(pfx + "_cind", m->cind, m->rptr[N]);
    dump(pfx + "_val", m->val, m->rptr[N]);
    long meta[4] = {N, m->M, bit, dbit};
    dump(pfx + "_meta", meta, 4);
}
template <typename T>
static void dump_csr_t(const std::string &pfx, void *p) {
    auto *m = reinterpret_cast<MCsrT<T> *>(p);
    int N = m->N;
    dump(pfx + "_rptr", m->rptr, N + 1);
    dump(pfx + "_cind", m->cind, m->rptr[N]);
    dump(pfx + "_val", m->val, m->rptr[N]);
    long meta[4] = {N, m->M, 0, 0};
    dump(pfx + "_meta", meta, 4);
}

// deterministic test vectors (not the reference's RNG; only inputs)
static uint64_t g_rng = 0x9E3779B97F4A7C15ull;
static uint64_t rnd() { g_rng ^= g_rng << 13; g_rng ^= g_rng >> 7; g_rng ^= g_rng << 17; return g_rng; }
static void rand_int(int *v, int n, int mag_bits) {
    for (int i = 0; i < n; i++) {
        long r = (long)(rnd() >> 11) & ((1L << mag_bits) - 1);
        v[i] = (int)(r - (1L << (mag_bits - 1)));
    }
}
static void rand_dbl(double *v, int n) {
    for (int i = 0; i < n; i++) v[i] = ((double)(rnd() >> 11) / 9007199254740992.0) * 2.0 - 1.0;
}

static double *read_vec(const char *path, int n) {
    double *b = utils::SafeMalloc<double>(n);
    FILE *f = fopen(path, "rb");
    if (!f || fread(b, sizeof(double), n, f) != (size_t)n) { fprintf(stderr, "bad b file %s\n", path); exit(2); }
    fclose(f);
    return b;
}

#define AMG_THETA 0.8

// ------------------------------------------------------------ integer hierarchy
// LDK: the smoother's LD class: 0 ldtri::CSRflex, 1 ldtri::BJCSRflex (block
// sizes dumped as _bjsize), 2 ldtri::MCCSRflex (colour sizes as _csize; the
// same field layout as BJCSRflex)
template <class SMO, int LDK, class AMG>
static void dump_int_hierarchy(AMG *iM, CSR<Fixed<30>> *iA) {
    auto *a0 = reinterpret_cast<MFixed *>(iA);
    dump_csr_int("A0", a0, 30, 0);
    int depth = iM->depth;
    dump_scalar_i("depth", depth);
    for (int l = 0; l <= depth; l++) {
        // smoother[l] is the smoother of level l (level 0 = fine grid); the
        // coarsest level (l == depth) uses the LU solver instead.
        if (l < depth) {
            SMO *s = iM->smoother[l];
            std::string p = "S" + std::to_string(l);
            if constexpr (LDK == 1 || LDK == 2) {
                auto *ld = reinterpret_cast<MBJ *>(s->LD);
                dump_csr_int(p + "_LD", ld, ld->bit, ld->dbit);
                dump(p + (LDK == 1 ? "_bjsize" : "_csize"), ld->bj_size, ld->bj_num + 1);
            } else {
                auto *ld = reinterpret_cast<MLD *>(s->LD);
                dump_csr_int(p + "_LD", ld, ld->bit, ld->dbit);
            }
            auto *u = reinterpret_cast<MFlex *>(s->U);
            dump_csr_int(p + "_U", u, u->bit, 0);
        }
    }
    for (int i = 0; i < depth; i++) {
        std::string p = "L" + std::to_string(i);
        if (i < depth - 1) {
            auto *ca = reinterpret_cast<MFlex *>(iM->C_A[i]);
            dump_csr_int(p + "_CA", ca, ca->bit, 0);
        }
        auto *ip = reinterpret_cast<MFlex *>(iM->Intrpl[i]);
        dump_csr_int(p + "_P", ip, ip->bit, 0);
        auto *it = reinterpret_cast<MFlex *>(iM->Intrpl_t[i]);
        dump_csr_int(p + "_R", it, it->bit, 0);
    }
    auto *lu = reinterpret_cast<MLUflex *>(iM->lu_solver);
    auto *L = reinterpret_cast<MLT *>(lu->L);
    auto *U = reinterpret_cast<MDU *>(lu->U);
    dump_csr_int("LU_L", L, L->bit, 0);
    dump_csr_int("LU_U", U, U->bit, U->dbit);
}

template <class SMO, class AMG>
static void int_kernel_tests(AMG *iM, CSR<Fixed<30>> *iA, int N, int bit) {
    // SpMV on level 0 and on every coarse operator, P and R; one sweep of every
    // smoother; V-cycle; the coarse LU solve.  Inputs have magnitude ~2^(bit+1).
    int mag = bit + 1 > 31 ? 31 : bit + 1;
    std::vector<int> x(N), y(N);
    rand_int(x.data(), N, mag);
    iA->SpMV(x.data(), y.data());
    dump("t_A0_in", x.data(), N);
    dump("t_A0_out", y.data(), N);
    int depth = iM->depth;
    for (int i = 0; i < depth; i++) {
        std::string p = "t_L" + std::to_string(i);
        auto *ip = reinterpret_cast<MFlex *>(iM->Intrpl[i]);
        std::vector<int> pin(ip->M), pout(ip->N);
        rand_int(pin.data(), ip->M, mag);
        iM->Intrpl[i]->SpMV(pin.data(), pout.data());
        dump(p + "_P_in", pin.data(), ip->M);
        dump(p + "_P_out", pout.data(), ip->N);
        auto *it = reinterpret_cast<MFlex *>(iM->Intrpl_t[i]);
        std::vector<int> rin(it->M), rout(it->N);
        rand_int(rin.data(), it->M, mag);
        iM->Intrpl_t[i]->SpMV(rin.data(), rout.data());
        dump(p + "_R_in", rin.data(), it->M);
        dump(p + "_R_out", rout.data(), it->N);
        if (i < depth - 1) {
            auto *ca = reinterpret_cast<MFlex *>(iM->C_A[i]);
            std::vector<int> cin(ca->M), cout_(ca->N);
            rand_int(cin.data(), ca->M, mag);
            iM->C_A[i]->SpMV(cin.data(), cout_.data());
            dump(p + "_CA_in", cin.data(), ca->M);
            dump(p + "_CA_out", cout_.data(), ca->N);
        }
    }
    for (int l = 0; l < depth; l++) {
        std::string p = "t_S" + std::to_string(l);
        SMO *s = iM->smoother[l];
        int n = s->LD->GetN();
        std::vector<int> in(n), out(n), out2(n);
        rand_int(in.data(), n, mag);
        s->LD->SpTRSV(in.data(), out.data());
        dump(p + "_LD_in", in.data(), n);
        dump(p + "_LD_out", out.data(), n);
        std::vector<int> uin(n), uout(n);
        rand_int(uin.data(), n, mag);
        s->U->SpMV(uin.data(), uout.data());
        dump(p + "_U_in", uin.data(), n);
        dump(p + "_U_out", uout.data(), n);
        // pre-smooth (isInited=false) then post-smooth (isInited=true) from that state
        s->Smooth(in.data(), out2.data(), false);
        dump(p + "_pre_out", out2.data(), n);
        s->Smooth(uin.data(), out2.data(), true);
        dump(p + "_post_out", out2.data(), n);
    }
    {
        auto *lu = reinterpret_cast<MLUflex *>(iM->lu_solver);
        auto *L = reinterpret_cast<MLT *>(lu->L);
        int n = L->N;
        std::vector<int> in(n), out(n);
        rand_int(in.data(), n, mag);
        iM->lu_solver->Solve(in.data(), out.data());
        dump("t_LU_in", in.data(), n);
        dump("t_LU_out", out.data(), n);
    }
    {
        std::vector<int> in(N), out(N);
        rand_int(in.data(), N, mag);
        iM->Precondition(in.data(), out.data());
        dump("t_V_in", in.data(), N);
        dump("t_V_out", out.data(), N);
    }
}

// ------------------------------------------------------------- FP hierarchies
template <typename T, class AMG>
static void dump_fp_hierarchy(const std::string &pfx, AMG *M) {
    int depth = M->depth;
    dump_scalar_i(pfx + "depth", depth);
    for (int l = 0; l < depth; l++) {
        auto *s = M->smoother[l];
        dump_csr_t<T>(pfx + "S" + std::to_string(l) + "_LD", s->LD);
        dump_csr_t<T>(pfx + "S" + std::to_string(l) + "_U", s->U);
    }
    for (int i = 0; i < depth; i++) {
        std::string p = pfx + "L" + std::to_string(i);
        if (i < depth - 1) dump_csr_t<T>(p + "_CA", M->C_A[i]);
        dump_csr_t<T>(p + "_P", M->Intrpl[i]);
        dump_csr_t<T>(p + "_R", M->Intrpl_t[i]);
    }
    auto *lu = reinterpret_cast<MLU<T> *>(M->lu_solver);
    dump_csr_t<T>(pfx + "LU_L", lu->L);
    dump_csr_t<T>(pfx + "LU_U", lu->U);
}

template <typename T, class AMG>
static void fp_kernel_tests(const std::string &pfx, AMG *M, int N) {
    std::vector<T> in(N), out(N);
    std::vector<double> tmp(N);
    rand_dbl(tmp.data(), N);
    for (int i = 0; i < N; i++) in[i] = (T)tmp[i];
    M->Precondition(in.data(), out.data());
    dump(pfx + "t_V_in", in.data(), N);
    dump(pfx + "t_V_out", out.data(), N);
    auto *s = M->smoother[0];
    std::vector<T> o2(N);
    s->LD->SpTRSV(in.data(), o2.data());
    dump(pfx + "t_S0_LD_out", o2.data(), N);
    auto *lu = reinterpret_cast<MLU<T> *>(M->lu_solver);
    auto *L = reinterpret_cast<MCsrT<T> *>(lu->L);
    int n = L->N;
    std::vector<T> lin(n), lout(n);
    for (int i = 0; i < n; i++) lin[i] = in[i];
    M->lu_solver->Solve(lin.data(), lout.data());
    dump(pfx + "t_LU_in", lin.data(), n);
    dump(pfx + "t_LU_out", lout.data(), n);
}

// ------------------------------------------------------------------- blas tests
static void blas_tests() {
    const int n = 4097;
    for (int bit = 20; bit <= 30; bit += 5) {
        std::string p = "blas_b" + std::to_string(bit);
        std::vector<int> x(n), y(n), y2(n), y3(n);
        rand_int(x.data(), n, bit + 1);
        rand_int(y.data(), n, bit + 1);
        dump(p + "_x", x.data(), n);
        dump(p + "_y", y.data(), n);
        long dot = blas1::int32::Dot(x.data(), y.data(), n, (int8_t)bit);
        long nrm = blas1::int32::Nrm2(x.data(), n, (int8_t)bit);
        long a = (long)(rnd() >> 33) - (1L << 30);
        y2 = y;
        blas1::int32::Axpy(a, x.data(), y2.data(), n, (int8_t)bit);
        y3 = x;
        blas1::int32::Scal(a, y3.data(), n, (int8_t)bit);
        std::vector<double> xd(n);
        rand_dbl(xd.data(), n);
        dump(p + "_xd_in", xd.data(), n);
        double ad = (double)(rnd() >> 11) / 9007199254740992.0 * 3.0 - 1.5;
        blas1::int32::Axpy_D(ad, x.data(), xd.data(), n, (int8_t)bit);
        long sc[3] = {dot, nrm, a};
        dump(p + "_scal", sc, 3);
        dump(p + "_ad", &ad, 1);
        dump(p + "_axpy", y2.data(), n);
        dump(p + "_scalv", y3.data(), n);
        dump(p + "_axpyd", xd.data(), n);
        // Givens generation / rotation on random int64 pairs
        const int ng = 64;
        std::vector<long> ga(ng), gb(ng), gc(ng), gs(ng), gr(ng), ra(ng), rb(ng);
        for (int i = 0; i < ng; i++) {
            ga[i] = (long)(rnd() >> 34) - (1L << 29);
            gb[i] = (long)(rnd() >> 35);
            long c, s;
            gr[i] = blas1::int32::Ggen(ga[i], gb[i], &c, &s, (int8_t)bit);
            gc[i] = c; gs[i] = s;
            long aa = (long)(rnd() >> 34) - (1L << 29), bb = (long)(rnd() >> 34) - (1L << 29);
            ra[i] = aa; rb[i] = bb;
        }
        dump(p + "_ga", ga.data(), ng); dump(p + "_gb", gb.data(), ng);
        dump(p + "_gc", gc.data(), ng); dump(p + "_gs", gs.data(), ng); dump(p + "_gr", gr.data(), ng);
        dump(p + "_ra", ra.data(), ng); dump(p + "_rb", rb.data(), ng);
        for (int i = 0; i < ng; i++) blas1::int32::Grot(gc[i], gs[i], &ra[i], &rb[i], (int8_t)bit);
        dump(p + "_ra_out", ra.data(), ng); dump(p + "_rb_out", rb.data(), ng);
        // lsqrt on a spread of magnitudes
        std::vector<long> lq(ng), lr(ng);
        for (int i = 0; i < ng; i++) { lq[i] = (long)(rnd() >> (1 + (i % 60))); lr[i] = blas1::int32::lsqrt<long>(lq[i]); }
        dump(p + "_lq", lq.data(), ng); dump(p + "_lr", lr.data(), ng);
    }
}

// --------------------------------------------------------------------- main
// usage:
//   ref_harness blas <outdir>
//   ref_harness solve <A.mtx> <b.f64> <outdir> <smoother 0 SOR|1 BlockSOR-40|2 JacobiSOR> <m> <what> <dump_cycle 0|1>
// where <what> is a comma list of: fp64 (FP64 solve), fp32 (FP32 solve),
// inth (int hierarchy + kernel tests), ints (int solve), dh / fh (dump the
// FP64 / FP32 hierarchies).
int main(int argc, char **argv) {
    if (argc >= 3 && std::string(argv[1]) == "blas") {
        g_out = argv[2];
        blas_tests();
        return 0;
    }
    if (argc != 9 || std::string(argv[1]) != "solve") {
        fprintf(stderr, "usage: ref_harness blas <outdir> | solve <A.mtx> <b.f64> <outdir> <smoother> <m> <int|fp64|fp32|all> <dump_cycle>\n");
        return 1;
    }
    const char *mtx = argv[2];
    g_out = argv[4];
    int smoother = atoi(argv[5]);
    int m = atoi(argv[6]);
    std::string what = "," + std::string(argv[7]) + ",";
    auto has = [&](const char *k) { return what.find("," + std::string(k) + ",") != std::string::npos; };
    int dump_cycle = atoi(argv[8]);

    CSRMat *Abase = io::ReadMM(mtx, true, false);
    int N = Abase->N;
    double *b = read_vec(argv[3], N);
    Abase->LMax1Scaling(b);
    dump("Ascaled_rptr", Abase->rptr, N + 1);
    dump("Ascaled_cind", Abase->cind, Abase->rptr[N]);
    dump("Ascaled_val", Abase->val, Abase->rptr[N]);
    dump("b_scaled", b, N);
    double nrm_b = blas1::Nrm2<double>(b, N);
    dump("nrm_b", &nrm_b, 1);

    auto dA = new CSR<double>(Abase);
    const int outer = 1000 / m;
    const double epsilon = 1.0e-10;
    double *x = utils::SafeMalloc<double>(N);
    double *r = utils::SafeMalloc<double>(N);
    auto sor_param = new SORParam(1.0, 1);
    auto hybrid_param = new BlockSORParam(1.0, 1, 40);

    auto explicit_res = [&](const std::string &tag) {
        dA->SpMV(x, r);
        blas1::Axpby<double>(1, b, -1, r, N);
        double nr = blas1::Nrm2<double>(r, N);
        printf("# [Res] : %e\n", nr / nrm_b);
        double rr = nr / nrm_b;
        dump(tag + "_res", &rr, 1);
        dump(tag + "_x", x, N);
    };

    using DSOR = SOR<ldtri::CSR<double>, CSR<double>>;
    using DBJ = BlockSOR<ldtri::BJCSR<double>, CSR<double>>;
    using FSOR = SOR<ldtri::CSR<float>, CSR<float>>;
    using FBJ = BlockSOR<ldtri::BJCSR<float>, CSR<float>>;
    using ISOR = SOR<ldtri::CSRflex, CSRflex>;
    using IBJ = BlockSORflex<ldtri::BJCSRflex, CSRflex>;
    using IJS = JacobiSORflex<ldtri::MCCSRflex, CSRflex>;

    Timer timer;
    // ---- FP64 preconditioner (also used by the bit rule, Work/main.cpp:153-161)
    Preconditioner<double> *M;
    if (smoother != 1) {  // SOR (also for the integer JacobiSOR case: the rule's V-cycle)
        auto *mm = new dfAMG<CSR<double>, DSOR, double>(Abase, dA, new AMGParam(20, AMG_THETA, 1, sor_param));
        if (has("dh")) dump_fp_hierarchy<double>("d_", mm);
        fp_kernel_tests<double>("d_", mm, N);
        M = mm;
    } else {
        auto *mm = new dfAMG<CSR<double>, DBJ, double>(Abase, dA, new AMGParam(20, AMG_THETA, 1, hybrid_param));
        fp_kernel_tests<double>("d_", mm, N);
        M = mm;
    }
    double *c = utils::SafeMalloc<double>(N);
    M->Precondition(b, c);
    double c_max = 0;
    for (int i = 0; i < N; i++) if (std::fabs(c[i]) > c_max) c_max = std::fabs(c[i]);
    int8_t bit = (c_max / nrm_b < 1) ? 29 : 31 - ((int)std::ceil(std::log2(int(c_max / nrm_b) + 1)) + 1);
    dump("c_bitrule", c, N);
    dump_scalar_i("bit", bit);
    printf("# bit %d\n", (int)bit);

    if (has("fp64")) {
        auto inner = new FGMRES<double>(dA, m, epsilon, M);
        auto solver = new Restarted(dA, inner, outer, epsilon);
        utils::Set<double>(0, x, N);
        timer.Restart();
        auto cv = solver->Solve(b, nrm_b, x);
        timer.Elapsed();
        printf("[Iter] : %d\n", cv.iter);
        dump_scalar_i("fp64_iter", cv.iter);
        explicit_res("fp64");
        delete solver; delete inner;
    }
    if (has("fp32")) {
        auto *fA = new CSR<float>(Abase);
        Preconditioner<float> *fM;
        if (smoother == 0) {
            auto *mm = new dfAMG<CSR<float>, FSOR, float>(Abase, fA, new AMGParam(20, AMG_THETA, 1, sor_param));
            if (has("fh")) dump_fp_hierarchy<float>("f_", mm);
            fp_kernel_tests<float>("f_", mm, N);
            fM = mm;
        } else {
            fM = new dfAMG<CSR<float>, FBJ, float>(Abase, fA, new AMGParam(20, AMG_THETA, 1, hybrid_param));
        }
        auto inner = new FGMRES<float>(fA, m, epsilon, fM);
        auto solver = new Restarted(dA, inner, outer, epsilon);
        utils::Set<double>(0, x, N);
        timer.Restart();
        auto cv = solver->Solve(b, nrm_b, x);
        timer.Elapsed();
        printf("[Iter] : %d\n", cv.iter);
        dump_scalar_i("fp32_iter", cv.iter);
        explicit_res("fp32");
    }
    if (has("inth") || has("ints")) {
        auto iA = new CSR<Fixed<30>>(Abase);
        if (smoother == 0) {
            auto *iM = new intAMGflex<CSRflex, CSRflex, ISOR>(Abase, iA, new AMGParam(20, AMG_THETA, 1, sor_param));
            dump_int_hierarchy<ISOR, 0>(iM, iA);
            int_kernel_tests<ISOR>(iM, iA, N, bit);
            auto inner = new FGMRESflex(iA, m, epsilon, iM, bit);
            if (dump_cycle) {
                // one Arnoldi cycle on r = b (x = 0), all internal state dumped
                utils::Set<double>(0, x, N);
                std::vector<double> rr(b, b + N);
                auto cv = inner->Solve(rr.data(), nrm_b, x);
                dump_scalar_i("cyc_iter", cv.iter);
                dump_scalar_i("cyc_conv", cv.isConverged);
                dump("cyc_V", inner->V, (size_t)N * (m + 1));
                dump("cyc_Z", inner->Z, (size_t)N * (m + 1));
                dump("cyc_H", inner->H, (size_t)(m + 1) * m);
                dump("cyc_c", inner->c, m);
                dump("cyc_s", inner->s, m);
                dump("cyc_e", inner->e, m + 1);
                dump("cyc_y", inner->y, m);
                dump("cyc_x", x, N);
            }
            if (has("ints")) {
                auto solver = new Restarted(dA, inner, outer, epsilon);
                utils::Set<double>(0, x, N);
                timer.Restart();
                auto cv = solver->Solve(b, nrm_b, x);
                timer.Elapsed();
                printf("[Iter] : %d\n", cv.iter);
                dump_scalar_i("int_iter", cv.iter);
                explicit_res("int");
            }
        } else if (smoother == 2) {
            auto *iM = new intAMGflex<CSRflex, CSRflex, IJS>(Abase, iA, new AMGParam(20, AMG_THETA, 1, sor_param));
            dump_int_hierarchy<IJS, 2>(iM, iA);
            int_kernel_tests<IJS>(iM, iA, N, bit);
            auto inner = new FGMRESflex(iA, m, epsilon, iM, bit);
            if (has("ints")) {
                auto solver = new Restarted(dA, inner, outer, epsilon);
                utils::Set<double>(0, x, N);
                timer.Restart();
                auto cv = solver->Solve(b, nrm_b, x);
                timer.Elapsed();
                printf("[Iter] : %d\n", cv.iter);
                dump_scalar_i("int_iter", cv.iter);
                explicit_res("int");
            }
        } else {
            auto *iM = new intAMGflex<CSRflex, CSRflex, IBJ>(Abase, iA, new AMGParam(20, AMG_THETA, 1, hybrid_param));
            dump_int_hierarchy<IBJ, 1>(iM, iA);
            int_kernel_tests<IBJ>(iM, iA, N, bit);
            auto inner = new FGMRESflex(iA, m, epsilon, iM, bit);
            if (has("ints")) {
                auto solver = new Restarted(dA, inner, outer, epsilon);
                utils::Set<double>(0, x, N);
                timer.Restart();
                auto cv = solver->Solve(b, nrm_b, x);
                timer.Elapsed();
                printf("[Iter] : %d\n", cv.iter);
                dump_scalar_i("int_iter", cv.iter);
                explicit_res("int");
            }
        }
    }
    return 0;
}
