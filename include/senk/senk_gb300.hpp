// C++ facade of the reference's solve-phase interface over the C ABI (sagb.h).
//
// The reference (suzuki-hpc/SC23-AD) is a header-only C++ library whose driver
// Work/main.cpp builds its objects from the `senk` namespace.  Compiling that
// driver with `-I include/senk` instead of `-I Library`, and linking
// libsagb.so, runs the same program on the GPU: the names, constructors and
// call order below are the ones the driver uses (Work/main.cpp:43-180), each
// implemented by the C ABI entry point that replaces it.  Errors print a
// message and exit, as the reference does (Library/utils/alloc.hpp:20-24,
// INTAMG.hpp:26-29).  Host pointers are accepted everywhere, as in the
// reference; the copies to and from the GPU happen inside the calls.
#ifndef SENK_GB300_FACADE_HPP
#define SENK_GB300_FACADE_HPP

#include <sys/time.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <iomanip>
#include <iostream>
#include <type_traits>

#include "../sagb.h"

namespace senk {

namespace detail {
inline void check(int code, const char *what) {
    if (code != SA_OK) {
        std::fprintf(stderr, "[sagb] %s: %s\n", what, sa_last_error());
        std::exit(1);
    }
}
// one context (GPU 0) for the whole program, like the reference's single process
inline sa_ctx context() {
    static sa_ctx c = nullptr;
    if (!c) check(sa_ctx_create(0, &c), "sa_ctx_create");
    return c;
}
}  // namespace detail

// ------------------------------------------------------------------ timer.hpp
inline double getTime() {
    struct timeval tv;
    gettimeofday(&tv, nullptr);
    return (double)tv.tv_sec + (double)tv.tv_usec * 1.0e-6;
}

// Prints "[Time] : <seconds>" like the reference (Work/Artwork/table.py parses it).
class Timer {
    double start_ = 0;

  public:
    Timer() { start_ = getTime(); }
    void Restart() { start_ = getTime(); }
    void Elapsed() {
        std::cout << "[Time] : " << std::fixed << std::setprecision(15) << getTime() - start_ << std::endl;
    }
};

// ---------------------------------------------------------------- utils.hpp
namespace utils {
template <typename T>
T *SafeMalloc(size_t n) {
    T *p = (T *)std::malloc(sizeof(T) * (n ? n : 1));
    if (!p) {
        std::fprintf(stderr, "Memory allocation failed.\n");
        std::exit(1);
    }
    return p;
}
template <typename T>
void Set(T v, T *x, int n) {
    for (int i = 0; i < n; i++) x[i] = v;
}
}  // namespace utils

// ----------------------------------------------------------------- blas1.hpp
namespace blas1 {
template <typename T>
T Nrm2(T *x, int n) {  // sequential sum, as blas1.hpp:63-70
    T s = 0;
    for (int i = 0; i < n; i++) s += x[i] * x[i];
    return std::sqrt(s);
}
template <typename T>
void Axpby(T a, T *x, T b, T *y, int n) {  // y = a x + b y
    for (int i = 0; i < n; i++) y[i] = a * x[i] + b * y[i];
}
}  // namespace blas1

// --------------------------------------------------------------- csrmat.hpp
// The fine matrix in host memory (the driver keeps ownership).
struct CSRMat {
    double *val = nullptr;
    int *cind = nullptr, *rptr = nullptr;
    int N = 0, M = 0;
    // CSRMat::LMax1Scaling (matrix/csrmat.hpp:70-80): rows and b divided by the row max
    void LMax1Scaling(double *b) {
        sa_hcsr h;
        detail::check(sa_hcsr_create(N, M, rptr, cind, val, &h), "LMax1Scaling");
        detail::check(sa_hcsr_lmax1_scaling(h, b), "LMax1Scaling");
        sa_csr_view v;
        detail::check(sa_hcsr_view(h, &v), "LMax1Scaling");
        const double *nv = (const double *)v.val;
        for (int64_t j = 0; j < v.nnz; j++) val[j] = nv[j];
        sa_hcsr_destroy(h);
    }
};

namespace io {
// io::ReadMM(path, true, false) (io/mm.hpp:24-98): expanded symmetric storage,
// explicit zeros dropped
inline CSRMat *ReadMM(const char *filename, bool is_expanded, bool has_zeros) {
    if (!is_expanded || has_zeros) {
        std::fprintf(stderr, "ReadMM: only (is_expanded = true, has_zeros = false) is provided\n");
        std::exit(1);
    }
    sa_hcsr h;
    detail::check(sa_hcsr_read_mm(filename, &h), "ReadMM");
    sa_csr_view v;
    detail::check(sa_hcsr_view(h, &v), "ReadMM");
    auto *A = new CSRMat();
    A->N = v.n;
    A->M = v.m;
    A->rptr = utils::SafeMalloc<int>(v.n + 1);
    A->cind = utils::SafeMalloc<int>(v.nnz);
    A->val = utils::SafeMalloc<double>(v.nnz);
    for (int i = 0; i <= v.n; i++) A->rptr[i] = v.rptr[i];
    for (int64_t j = 0; j < v.nnz; j++) {
        A->cind[j] = v.cind[j];
        A->val[j] = ((const double *)v.val)[j];
    }
    sa_hcsr_destroy(h);
    return A;
}
}  // namespace io

// ----------------------------------------------------------- spmat.hpp types
template <int B>
struct Fixed {};  // Fix<32, B> element tag (CSR<Fixed<30>>)

template <typename T>
class SpMat {
  public:
    sa_mat h = nullptr;
    int N = 0;
    virtual ~SpMat() {
        if (h) sa_mat_destroy(h);
    }
    int GetN() { return N; }
    virtual void SpMV(T *in, T *out) { detail::check(sa_spmv(detail::context(), h, in, out), "SpMV"); }
};

template <typename T>
class CSR : public SpMat<T> {
  public:
    explicit CSR(CSRMat *A) {
        static_assert(std::is_same<T, double>::value || std::is_same<T, float>::value, "CSR<double> or CSR<float>");
        this->N = A->N;
        const int kind = std::is_same<T, double>::value ? SA_MAT_F64 : SA_MAT_F32;
        detail::check(sa_mat_create(detail::context(), kind, 0, A->N, A->M, A->rptr, A->cind, A->val, &this->h),
                      "CSR");
    }
};

template <int B>
class CSR<Fixed<B>> : public SpMat<int> {
  public:
    explicit CSR(CSRMat *A) {
        this->N = A->N;
        detail::check(sa_mat_create(detail::context(), SA_MAT_FIXED, B, A->N, A->M, A->rptr, A->cind, A->val,
                                    &this->h),
                      "CSR<Fixed>");
    }
};

// Operator and smoother type tags (the class template arguments of the driver)
class CSRflex {};
namespace ldtri {
class CSRflex {};
class BJCSRflex {};
class MCCSRflex {};
template <typename T>
class CSR {};
template <typename T>
class BJCSR {};
}  // namespace ldtri
template <typename LD, typename U>
class SOR {};
template <typename LD, typename U>
class BlockSOR {};
template <typename LD, typename U>
class BlockSORflex {};
template <typename LD, typename U>
class JacobiSORflex {};  // smoother/stationary.hpp:564-676 (with SORParam)

namespace detail {
template <typename S>
struct is_jacobi_sor : std::false_type {};
template <typename LD, typename U>
struct is_jacobi_sor<JacobiSORflex<LD, U>> : std::true_type {};
}  // namespace detail

// ---------------------------------------------------------- parameters.hpp
struct SmootherParam {
    virtual ~SmootherParam() {}
};
struct SORParam : public SmootherParam {
    double omega;
    int iter;
    SORParam(double _omega, int _iter) : omega(_omega), iter(_iter) {}
};
struct BlockSORParam : public SmootherParam {
    double omega;
    int iter, b_num;
    BlockSORParam(double _omega, int _iter, int _b_num) : omega(_omega), iter(_iter), b_num(_b_num) {}
};
struct PreconditionerParam {
    virtual ~PreconditionerParam() {}
};
struct AMGParam : public PreconditionerParam {
    int level;
    double theta;
    int cycle;
    SmootherParam *param;
    AMGParam(int _level, double _theta, int _cycle, SmootherParam *_param)
        : level(_level), theta(_theta), cycle(_cycle), param(_param) {}
};

// ------------------------------------------------------------ INTAMG.hpp
template <typename T>
class Preconditioner {
  public:
    sa_amg h = nullptr;
    virtual ~Preconditioner() {
        if (h) sa_amg_destroy(h);
    }
    virtual void Precondition(T *in, T *out) {
        detail::check(sa_amg_precondition(detail::context(), h, in, out), "Precondition");
    }
};

namespace detail {
inline sa_amg_params amg_params(PreconditionerParam *p) {
    auto *ap = dynamic_cast<AMGParam *>(p);
    if (!ap || ap->cycle != 1) {
        std::fprintf(stderr, "AMG: an AMGParam with the V-cycle (cycle = 1) is expected\n");
        std::exit(1);
    }
    sa_amg_params q;
    sa_amg_params_default(&q);
    q.max_levels = ap->level;
    q.theta = ap->theta;
    if (auto *s = dynamic_cast<SORParam *>(ap->param)) {
        q.omega = s->omega;
        q.smooth_iter = s->iter;
        q.smoother_blocks = 0;
    } else if (auto *s = dynamic_cast<BlockSORParam *>(ap->param)) {
        q.omega = s->omega;
        q.smooth_iter = s->iter;
        q.smoother_blocks = s->b_num;
    } else {
        std::fprintf(stderr, "AMG: SORParam or BlockSORParam expected\n");
        std::exit(1);
    }
    return q;
}
}  // namespace detail

// dfAMG<SpMatClass, Smoother, T> (INTAMG.hpp:13-134): FP64 / FP32 V-cycle
template <typename SpMatClass, typename Smoother, typename T>
class dfAMG : public Preconditioner<T> {
  public:
    dfAMG(CSRMat *A, SpMat<T> *, PreconditionerParam *p) {
        const sa_amg_params q = detail::amg_params(p);
        const int prec = std::is_same<T, double>::value ? SA_F64 : SA_F32;
        detail::check(sa_amg_create(detail::context(), prec, &q, A->N, A->rptr, A->cind, A->val, &this->h), "dfAMG");
    }
};

// intAMGflex<C, I, Smoother> (INTAMG.hpp:136-293): integer V-cycle
template <typename C, typename I, typename Smoother>
class intAMGflex : public Preconditioner<int> {
  public:
    intAMGflex(CSRMat *A, SpMat<int> *, PreconditionerParam *p) {
        sa_amg_params q = detail::amg_params(p);
        if (detail::is_jacobi_sor<Smoother>::value) q.multicolor = 2;  // JacobiSORflex: 1200-row chunks
        detail::check(sa_amg_create(detail::context(), SA_INT, &q, A->N, A->rptr, A->cind, A->val, &this->h),
                      "intAMGflex");
    }
};

// ------------------------------------------------------ gmres.hpp / irsolver.hpp
struct Converge {
    bool isConverged = false;
    int iter = 0;
    Converge() {}
    Converge(bool c, int it) : isConverged(c), iter(it) {}
};

class Solver {
  public:
    virtual ~Solver() {}
    virtual Converge Solve(double *b, double nrm_b, double *x) = 0;
};

// The inner solvers only carry their arguments; Restarted builds the GPU solver.
class InnerSolver {
  public:
    int precision = SA_F64;
    sa_mat A = nullptr;
    sa_amg M = nullptr;
    int m = 30;
    double eps = 1e-10;
    int bit = 29;
    virtual ~InnerSolver() {}
};

template <typename T>
class FGMRES : public InnerSolver {
  public:
    FGMRES(SpMat<T> *A_, int m_, double eps_, Preconditioner<T> *M_) {
        precision = std::is_same<T, double>::value ? SA_F64 : SA_F32;
        A = A_->h;
        M = M_->h;
        m = m_;
        eps = eps_;
    }
};

class FGMRESflex : public InnerSolver {
  public:
    FGMRESflex(SpMat<int> *A_, int m_, double eps_, Preconditioner<int> *M_, int8_t bit_) {
        precision = SA_INT;
        A = A_->h;
        M = M_->h;
        m = m_;
        eps = eps_;
        bit = bit_;
    }
};

// Restarted (irsolver.hpp:27-43) around the inner solver; prints the
// reference's per-iteration "# [j] res" lines.
class Restarted : public Solver {
    sa_solver S_ = nullptr;

  public:
    Restarted(SpMat<double> *dA, InnerSolver *inner, int outer, double eps) {
        sa_solver_params p;
        sa_solver_params_default(&p);
        p.m = inner->m;
        p.eps = eps;
        p.max_outer = outer;
        p.frac_bits = inner->bit;
        p.verbose = 1;
        detail::check(sa_solver_create(detail::context(), inner->precision, dA->h, inner->A, inner->M, &p, &S_),
                      "Restarted");
    }
    ~Restarted() override {
        if (S_) sa_solver_destroy(S_);
    }
    Converge Solve(double *b, double nrm_b, double *x) override {
        int it = 0, conv = 0;
        detail::check(sa_solver_solve(S_, b, nrm_b, x, &it, &conv), "Solve");
        return Converge(conv != 0, it);
    }
};

}  // namespace senk

#endif
