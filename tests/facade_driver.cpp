// A driver written against the senk facade (include/senk): reads a Matrix
// Market file, scales it, builds the FP64, FP32 or integer AMG preconditioner,
// picks F by the reference's rule and solves with Restarted(FGMRES<double>),
// Restarted(FGMRES<float>) or Restarted(FGMRESflex), as Work/main.cpp does.
// Arguments: <matrix.mtx> <0: FP64, 1: FP32-mixed, 2: int, 3: int with JacobiSORflex> <m> [b.f64], where
// the optional file holds the unscaled right-hand side as raw FP64 values.
// Prints "[Iter] : n" and "# [Res] : r" like the reference's driver.
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "blas/blas1.hpp"
#include "io/mm.hpp"
#include "preconditioner/INTAMG.hpp"
#include "solver/gmres.hpp"
#include "solver/irsolver.hpp"
#include "timer.hpp"

using namespace senk;

int main(int argc, char **argv) {
    if (argc != 4 && argc != 5) return 1;
    CSRMat *A = io::ReadMM(argv[1], true, false);
    const int kind = std::atoi(argv[2]), m = std::atoi(argv[3]);
    const int N = A->N;
    double *b = utils::SafeMalloc<double>(N);
    if (argc == 5) {
        FILE *f = std::fopen(argv[4], "rb");
        if (!f || std::fread(b, sizeof(double), N, f) != (size_t)N) return 2;
        std::fclose(f);
    } else {
        for (int i = 0; i < N; i++) b[i] = 1.0 + 0.5 * std::sin(0.1 * i);
    }
    A->LMax1Scaling(b);
    const double nrm_b = blas1::Nrm2<double>(b, N);
    auto *dA = new CSR<double>(A);
    double *x = utils::SafeMalloc<double>(N);
    utils::Set<double>(0, x, N);
    auto *sor = new SORParam(1.0, 1);
    auto *param = new AMGParam(20, 0.8, 1, sor);
    Converge cv;
    auto *timer = new Timer();
    if (kind == 0) {
        auto *M = new dfAMG<CSR<double>, SOR<ldtri::CSR<double>, CSR<double>>, double>(A, dA, param);
        auto *inner = new FGMRES<double>(dA, m, 1e-10, M);
        auto *S = new Restarted(dA, inner, 1000 / m, 1e-10);
        timer->Restart();
        cv = S->Solve(b, nrm_b, x);
        timer->Elapsed();
        delete S;
        delete M;
    } else if (kind == 1) {
        auto *fA = new CSR<float>(A);
        auto *M = new dfAMG<CSR<float>, SOR<ldtri::CSR<float>, CSR<float>>, float>(A, fA, param);
        auto *inner = new FGMRES<float>(fA, m, 1e-10, M);
        auto *S = new Restarted(dA, inner, 1000 / m, 1e-10);
        timer->Restart();
        cv = S->Solve(b, nrm_b, x);
        timer->Elapsed();
        delete S;
        delete M;
        delete fA;
    } else {
        auto *iA = new CSR<Fixed<30>>(A);
        auto *M = new dfAMG<CSR<double>, SOR<ldtri::CSR<double>, CSR<double>>, double>(A, dA, param);
        Preconditioner<int> *iM;
        if (kind == 3) iM = new intAMGflex<CSRflex, CSRflex, JacobiSORflex<ldtri::MCCSRflex, CSRflex>>(A, iA, param);
        else iM = new intAMGflex<CSRflex, CSRflex, SOR<ldtri::CSRflex, CSRflex>>(A, iA, param);
        double *c = utils::SafeMalloc<double>(N);
        M->Precondition(b, c);
        double cmax = 0;
        for (int i = 0; i < N; i++) cmax = std::fmax(cmax, std::fabs(c[i]));
        const double q = cmax / nrm_b;
        const int8_t bit = q < 1 ? 29 : 31 - ((int)std::ceil(std::log2(int(q) + 1)) + 1);
        delete M;
        auto *inner = new FGMRESflex(iA, m, 1e-10, iM, bit);
        auto *S = new Restarted(dA, inner, 1000 / m, 1e-10);
        timer->Restart();
        cv = S->Solve(b, nrm_b, x);
        timer->Elapsed();
        delete S;
        delete iM;
        delete iA;
        std::free(c);
    }
    std::printf("[Iter] : %d\n", cv.iter);
    double *r = utils::SafeMalloc<double>(N);
    dA->SpMV(x, r);
    blas1::Axpby<double>(1, b, -1, r, N);
    std::printf("# [Res] : %e\n", blas1::Nrm2<double>(r, N) / nrm_b);
    return 0;
}
