// Device AMG hierarchy and the V-cycle.
//
// intAMGflex::Precondition (preconditioner/INTAMG.hpp:269-293) and
// dfAMG::Precondition (INTAMG.hpp:108-133), with the SOR/BlockSOR smoothing
// of smoother/stationary.hpp (415-430, 997-1012, 238-255).  Pairs of reference
// calls that read the same data are fused into one kernel:
//   A*out then Sub(in, r)           -> one residual SpMV (SPMV_RESID)
//   P*xx then Add(rr, xx)           -> one prolongate-and-add SpMV (SPMV_ADD)
//   U*out then Axpby(1, in, -1, t)  -> one residual SpMV with U
#include "../sagb_internal.hpp"
#include "common.cuh"

namespace sagb {

void DevAmg::release() {
    A0.release();
    for (auto &m : CA) m.release();
    for (auto &m : P) m.release();
    for (auto &m : R) m.release();
    for (auto &m : U) m.release();
    for (auto &t : LD) t.release();
    LU.release();
    dfree(r);
    for (void *p : rr) dfree(p);
    for (void *p : ee) dfree(p);
    for (void *p : xx) dfree(p);
    for (void *p : tmp) dfree(p);
    r = nullptr;
    rr.clear(); ee.clear(); xx.clear(); tmp.clear();
}

static void alloc_vectors(DevAmg &M) {
    const size_t es = vt_size(M.vt);
    M.r = dmalloc(es * (size_t)M.A0.n);
    for (int i = 0; i < M.depth; i++) {
        const int len = M.R[i].n;
        M.rr.push_back(dmalloc(es * (size_t)len));
        M.ee.push_back(dmalloc(es * (size_t)len));
        M.xx.push_back(dmalloc(es * (size_t)len));
        SAGB_CUDA(cudaMemset(M.xx.back(), 0, es * (size_t)len));
    }
    for (int l = 0; l < M.depth; l++) M.tmp.push_back(dmalloc(es * (size_t)M.LD[l].n));
}

std::unique_ptr<DevAmg> upload_amg_int(Ctx &c, std::shared_ptr<IntHierarchy> h) {
    auto M = std::make_unique<DevAmg>();
    M->vt = VT_I32;
    M->depth = h->depth;
    M->smooth_iter = h->smooth_iter;
    M->A0 = upload_csr_i32(h->A0);
    for (auto &m : h->CA) M->CA.push_back(upload_csr_i32(m));
    for (auto &m : h->P) M->P.push_back(upload_csr_i32(m));
    for (auto &m : h->R) M->R.push_back(upload_csr_i32(m));
    for (auto &m : h->U) M->U.push_back(upload_csr_i32(m));
    for (int l = 0; l < h->depth; l++) {
        const CsrI &m = h->LD[l];
        const int *hint = h->colour[l].empty() ? nullptr : h->colour[l].data();
        M->LD.push_back(
            upload_tri(c, m.n, m.rptr.data(), m.cind.data(), m.val.data(), VT_I32, TRI_LD, m.bit, m.dbit, hint));
    }
    M->nbj = h->bj.empty() || h->bj[0].empty() ? 0 : (int)h->bj[0].size() - 1;
    M->LU = upload_dense_lu(h->LUL.rptr.data(), h->LUL.cind.data(), h->LUL.val.data(), h->LUU.rptr.data(),
                            h->LUU.cind.data(), h->LUU.val.data(), h->LUL.n, VT_I32, h->LUL.bit, h->LUU.bit,
                            h->LUU.dbit);
    alloc_vectors(*M);
    M->hi = h;
    return M;
}

template <typename T>
static std::unique_ptr<DevAmg> upload_amg_fp(Ctx &c, const FpHierarchy<T> &h, int vt) {
    auto M = std::make_unique<DevAmg>();
    M->vt = vt;
    M->depth = h.depth;
    M->smooth_iter = h.smooth_iter;
    M->A0 = upload_csr_fp<T>(h.A0);
    for (auto &m : h.CA) M->CA.push_back(upload_csr_fp<T>(m));
    for (auto &m : h.P) M->P.push_back(upload_csr_fp<T>(m));
    for (auto &m : h.R) M->R.push_back(upload_csr_fp<T>(m));
    for (auto &m : h.U) M->U.push_back(upload_csr_fp<T>(m));
    for (int l = 0; l < h.depth; l++) {
        const auto &m = h.LD[l];
        const int *hint = h.colour[l].empty() ? nullptr : h.colour[l].data();
        M->LD.push_back(upload_tri(c, m.n, m.rptr.data(), m.cind.data(), m.val.data(), vt, TRI_LD, 0, 0, hint));
    }
    M->nbj = h.bj.empty() || h.bj[0].empty() ? 0 : (int)h.bj[0].size() - 1;
    M->LU = upload_dense_lu(h.LUL.rptr.data(), h.LUL.cind.data(), h.LUL.val.data(), h.LUU.rptr.data(),
                            h.LUU.cind.data(), h.LUU.val.data(), h.LUL.n, vt, 0, 0, 0);
    alloc_vectors(*M);
    return M;
}

std::unique_ptr<DevAmg> upload_amg_f64(Ctx &c, std::shared_ptr<FpHierarchy<double>> h) {
    auto M = upload_amg_fp<double>(c, *h, VT_F64);
    M->hd = h;
    return M;
}
std::unique_ptr<DevAmg> upload_amg_f32(Ctx &c, std::shared_ptr<FpHierarchy<float>> h) {
    auto M = upload_amg_fp<float>(c, *h, VT_F32);
    M->hf = h;
    return M;
}

void smooth(Ctx &c, DevAmg &M, int l, const void *in, void *out, bool inited) {
    int k0 = 0;
    if (!inited) {
        trsv(c, M.LD[l], in, out);
        k0 = 1;
    }
    for (int k = k0; k < M.smooth_iter; k++) {
        spmv(c, M.U[l], out, M.tmp[l], SPMV_RESID, in);
        trsv(c, M.LD[l], M.tmp[l], out);
    }
}

void vcycle(Ctx &c, DevAmg &M, const void *in, void *out) {
    PrecFlags pf(c);
    const int D = M.depth;
    smooth(c, M, 0, in, out, false);
    spmv(c, M.A0, out, M.r, SPMV_RESID, in);
    spmv(c, M.R[0], M.r, M.ee[0]);
    for (int i = 0; i < D - 1; i++) {
        smooth(c, M, i + 1, M.ee[i], M.xx[i], false);
        spmv(c, M.CA[i], M.xx[i], M.rr[i], SPMV_RESID, M.ee[i]);
        spmv(c, M.R[i + 1], M.rr[i], M.ee[i + 1]);
    }
    lu_solve(c, M.LU, M.ee[D - 1], M.xx[D - 1]);
    for (int i = D - 2; i >= 0; i--) {
        spmv(c, M.P[i + 1], M.xx[i + 1], M.xx[i], SPMV_ADD);
        smooth(c, M, i + 1, M.ee[i], M.xx[i], true);
    }
    spmv(c, M.P[0], M.xx[0], out, SPMV_ADD);
    smooth(c, M, 0, in, out, true);
}

}  // namespace sagb
