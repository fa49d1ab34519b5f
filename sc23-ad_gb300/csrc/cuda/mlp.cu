// The learned fractional-bit selector: a 3-layer FP32 MLP (in -> H -> H -> out,
// ReLU after the two hidden layers) trained and evaluated by these kernels.
//
// The reference picks F_G by a fixed rule (Work/main.cpp:153-161) or by a
// manual sweep (Work/sub.cpp:36-102, Work/run_sub.sh); it has no learned part,
// so this file has no reference counterpart.  The network maps matrix features
// to one predicted cost per candidate F (log2 of the iteration count of the
// integer solver); the selector takes the argmin.
//
// Every kernel reduces in a fixed order (no atomics), so training is
// reproducible run to run.  Parameter layout (one flat float array):
//   W1[H][I] b1[H] W2[H][H] b2[H] W3[O][H] b3[O]
#include <cmath>
#include <cstring>
#include <vector>

#include "../sagb_internal.hpp"
#include "common.cuh"

namespace sagb {

constexpr int kTile = 16;

// Y[b][n] = act(sum_k X[b][k] W[n][k] + bias[n]), k summed in increasing order.
__global__ void k_dense_fwd(const float *__restrict__ X, const float *__restrict__ W,
                            const float *__restrict__ bias, float *__restrict__ Y, int B, int K, int N, int relu) {
    __shared__ float sx[kTile][kTile + 1], sw[kTile][kTile + 1];
    const int tb = threadIdx.y, tn = threadIdx.x;
    const int b = blockIdx.y * kTile + tb, n = blockIdx.x * kTile + tn;
    float acc = 0.f;
    for (int k0 = 0; k0 < K; k0 += kTile) {
        const int kx = k0 + tn;
        sx[tb][tn] = (b < B && kx < K) ? X[(size_t)b * K + kx] : 0.f;
        const int nw = blockIdx.x * kTile + tb;
        sw[tb][tn] = (nw < N && kx < K) ? W[(size_t)nw * K + kx] : 0.f;
        __syncthreads();
        const int kk = min(kTile, K - k0);
        for (int t = 0; t < kk; t++) acc = __fmaf_rn(sx[tb][t], sw[tn][t], acc);
        __syncthreads();
    }
    if (b < B && n < N) {
        float y = acc + bias[n];
        if (relu) y = fmaxf(y, 0.f);
        Y[(size_t)b * N + n] = y;
    }
}

// dX[b][k] = (sum_n dY[b][n] W[n][k]) * (A[b][k] > 0), n in increasing order.
// A is the layer's input activation (post-ReLU), so the product is the
// gradient with respect to the previous layer's pre-activation.
__global__ void k_dense_bwd_x(const float *__restrict__ dY, const float *__restrict__ W,
                              const float *__restrict__ A, float *__restrict__ dX, int B, int N, int K) {
    __shared__ float sd[kTile][kTile + 1], sw[kTile][kTile + 1];
    const int tb = threadIdx.y, tk = threadIdx.x;
    const int b = blockIdx.y * kTile + tb, k = blockIdx.x * kTile + tk;
    float acc = 0.f;
    for (int n0 = 0; n0 < N; n0 += kTile) {
        const int nd = n0 + tk;
        sd[tb][tk] = (b < B && nd < N) ? dY[(size_t)b * N + nd] : 0.f;
        const int nw = n0 + tb;
        sw[tb][tk] = (nw < N && k < K) ? W[(size_t)nw * K + k] : 0.f;
        __syncthreads();
        const int nn = min(kTile, N - n0);
        for (int t = 0; t < nn; t++) acc = __fmaf_rn(sd[tb][t], sw[t][tk], acc);
        __syncthreads();
    }
    if (b < B && k < K) dX[(size_t)b * K + k] = A[(size_t)b * K + k] > 0.f ? acc : 0.f;
}

// dW[n][k] = sum_b dY[b][n] X[b][k]; db[n] = sum_b dY[b][n]; b in increasing order.
__global__ void k_dense_bwd_w(const float *__restrict__ dY, const float *__restrict__ X, float *__restrict__ dW,
                              float *__restrict__ db, int B, int N, int K) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < N * K) {
        const int n = idx / K, k = idx - n * K;
        float acc = 0.f;
        for (int b = 0; b < B; b++) acc = __fmaf_rn(dY[(size_t)b * N + n], X[(size_t)b * K + k], acc);
        dW[idx] = acc;
    } else if (idx < N * K + N) {
        const int n = idx - N * K;
        float acc = 0.f;
        for (int b = 0; b < B; b++) acc += dY[(size_t)b * N + n];
        db[n] = acc;
    }
}

// Masked mean squared error over one batch (one block):
//   L = sum M (Y - T)^2 / sum M,  dY = 2 M (Y - T) / sum M.
__global__ void k_mse(const float *__restrict__ Y, const float *__restrict__ T, const float *__restrict__ M,
                      float *__restrict__ dY, int count, float *__restrict__ loss) {
    __shared__ float sh[32];
    __shared__ float s_tot;
    float m = 0.f;
    for (int i = threadIdx.x; i < count; i += blockDim.x) m += M[i];
    // fixed-order block sum: warp shuffles, then warp 0 over the warp sums
    auto bsum = [&](float v) {
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
        __syncthreads();
        if (threadIdx.x == 0) {
            float t = 0.f;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
            s_tot = t;
        }
        __syncthreads();
        const float r = s_tot;
        __syncthreads();
        return r;
    };
    const float msum = bsum(m);
    const float inv = msum > 0.f ? 1.f / msum : 0.f;
    float e = 0.f;
    for (int i = threadIdx.x; i < count; i += blockDim.x) {
        const float d = Y[i] - T[i];
        e += M[i] * d * d;
        dY[i] = 2.f * M[i] * d * inv;
    }
    const float esum = bsum(e);
    if (threadIdx.x == 0) *loss = esum * inv;
}

// Adam (Kingma & Ba 2015) with bias correction; t is the 1-based step count.
__global__ void k_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m1,
                       float *__restrict__ m2, int n, float lr, float beta1, float beta2, float eps, float bc1,
                       float bc2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float a = beta1 * m1[i] + (1.f - beta1) * gi;
    const float v = beta2 * m2[i] + (1.f - beta2) * gi * gi;
    m1[i] = a;
    m2[i] = v;
    const float mh = a / bc1, vh = v / bc2;
    w[i] -= lr * mh / (sqrtf(vh) + eps);
}

// Xn[b][k] = (X[src(b)][k] - mu[k]) / sd[k]; rows gathered through perm (or
// taken in order when perm is null), targets and masks gathered alike.
__global__ void k_gather_norm(const float *__restrict__ X, const float *__restrict__ T, const float *__restrict__ M,
                              const int *__restrict__ perm, int off, int B, int I, int O,
                              const float *__restrict__ mu, const float *__restrict__ sd, float *__restrict__ Xb,
                              float *__restrict__ Tb, float *__restrict__ Mb) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const int b = idx / (I + O), r = idx - b * (I + O);
    if (b >= B) return;
    const int s = perm ? perm[off + b] : off + b;
    if (r < I) {
        Xb[(size_t)b * I + r] = (X[(size_t)s * I + r] - mu[r]) / sd[r];
    } else if (T) {
        const int o = r - I;
        Tb[(size_t)b * O + o] = T[(size_t)s * O + o];
        Mb[(size_t)b * O + o] = M[(size_t)s * O + o];
    }
}

// ------------------------------------------------------------------ host side

Mlp::Mlp(int in, int hidden, int out, uint64_t seed) : nin(in), hid(hidden), nout(out) {
    if (in < 1 || hidden < 1 || out < 1 || in > 4096 || hidden > 4096 || out > 4096)
        throw CudaError{"invalid MLP shape"};
    const size_t np = nparams();
    // He-uniform initialisation from a splitmix64 stream (identical on every host)
    std::vector<float> w(np, 0.f);
    uint64_t st = seed;
    auto next = [&]() {
        uint64_t z = (st += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    auto fill = [&](size_t off, int rows, int cols) {
        const double lim = std::sqrt(6.0 / cols);
        for (size_t i = 0; i < (size_t)rows * cols; i++) w[off + i] = (float)((2.0 * next() - 1.0) * lim);
    };
    fill(off_w1(), hid, nin);
    fill(off_w2(), hid, hid);
    fill(off_w3(), nout, hid);
    p = (float *)dmalloc(np * 4 * sizeof(float));
    g = p + np;
    m1 = g + np;
    m2 = m1 + np;
    SAGB_CUDA(cudaMemcpy(p, w.data(), np * sizeof(float), cudaMemcpyHostToDevice));
    SAGB_CUDA(cudaMemset(g, 0, 3 * np * sizeof(float)));
    std::vector<float> mu(nin, 0.f), sd(nin, 1.f);
    norm = (float *)dmalloc(2 * nin * sizeof(float));
    SAGB_CUDA(cudaMemcpy(norm, mu.data(), nin * sizeof(float), cudaMemcpyHostToDevice));
    SAGB_CUDA(cudaMemcpy(norm + nin, sd.data(), nin * sizeof(float), cudaMemcpyHostToDevice));
}

Mlp::~Mlp() {
    dfree(p);
    dfree(norm);
    dfree(ws);
    dfree(data);
    dfree(perm_d);
}

void Mlp::reserve(int B) {
    if (B <= ws_batch) return;
    dfree(ws);
    // Xb, A1, A2, Y, Tb, Mb, dY, d2, d1, loss
    const size_t n = (size_t)B * (nin + 4 * hid + 4 * nout) + 1;
    ws = (float *)dmalloc(n * sizeof(float));
    ws_batch = B;
}

void Mlp::forward_batch(Ctx &c, int B) {
    float *Xb = ws, *A1 = Xb + (size_t)ws_batch * nin, *A2 = A1 + (size_t)ws_batch * hid,
          *Y = A2 + (size_t)ws_batch * hid;
    const dim3 blk(kTile, kTile);
    auto grid = [&](int n) { return dim3((n + kTile - 1) / kTile, (B + kTile - 1) / kTile); };
    k_dense_fwd<<<grid(hid), blk, 0, c.stream>>>(Xb, p + off_w1(), p + off_b1(), A1, B, nin, hid, 1);
    k_dense_fwd<<<grid(hid), blk, 0, c.stream>>>(A1, p + off_w2(), p + off_b2(), A2, B, hid, hid, 1);
    k_dense_fwd<<<grid(nout), blk, 0, c.stream>>>(A2, p + off_w3(), p + off_b3(), Y, B, hid, nout, 0);
    c.launches += 3;
}

void Mlp::backward_batch(Ctx &c, int B) {
    float *Xb = ws, *A1 = Xb + (size_t)ws_batch * nin, *A2 = A1 + (size_t)ws_batch * hid,
          *Y = A2 + (size_t)ws_batch * hid, *Tb = Y + (size_t)ws_batch * nout, *Mb = Tb + (size_t)ws_batch * nout,
          *dY = Mb + (size_t)ws_batch * nout, *d2 = dY + (size_t)ws_batch * nout, *d1 = d2 + (size_t)ws_batch * hid,
          *loss = d1 + (size_t)ws_batch * hid;
    k_mse<<<1, 1024, 0, c.stream>>>(Y, Tb, Mb, dY, B * nout, loss);
    const dim3 blk(kTile, kTile);
    auto gridx = [&](int k) { return dim3((k + kTile - 1) / kTile, (B + kTile - 1) / kTile); };
    auto gw = [&](int n, int k) { return (n * k + n + 255) / 256; };
    k_dense_bwd_w<<<gw(nout, hid), 256, 0, c.stream>>>(dY, A2, g + off_w3(), g + off_b3(), B, nout, hid);
    k_dense_bwd_x<<<gridx(hid), blk, 0, c.stream>>>(dY, p + off_w3(), A2, d2, B, nout, hid);
    k_dense_bwd_w<<<gw(hid, hid), 256, 0, c.stream>>>(d2, A1, g + off_w2(), g + off_b2(), B, hid, hid);
    k_dense_bwd_x<<<gridx(hid), blk, 0, c.stream>>>(d2, p + off_w2(), A1, d1, B, hid, hid);
    k_dense_bwd_w<<<gw(hid, nin), 256, 0, c.stream>>>(d1, Xb, g + off_w1(), g + off_b1(), B, hid, nin);
    c.launches += 6;
}

float *Mlp::loss_slot() { return ws + (size_t)ws_batch * (nin + 4 * hid + 4 * nout); }

void Mlp::set_norm(const float *mu, const float *sd) {
    for (int i = 0; i < nin; i++)
        if (!(sd[i] > 0.f)) throw CudaError{"feature scale must be positive"};
    SAGB_CUDA(cudaMemcpy(norm, mu, nin * sizeof(float), cudaMemcpyHostToDevice));
    SAGB_CUDA(cudaMemcpy(norm + nin, sd, nin * sizeof(float), cudaMemcpyHostToDevice));
}

void Mlp::load(Ctx &c, const float *X, const float *T, const float *M, int n) {
    const size_t bytes = (size_t)n * (nin + 2 * nout) * sizeof(float);
    if (n > data_n) {
        dfree(data);
        data = (float *)dmalloc(bytes);
        data_n = n;
    }
    SAGB_CUDA(cudaMemcpyAsync(data, X, (size_t)n * nin * sizeof(float), cudaMemcpyDefault, c.stream));
    if (T) {
        SAGB_CUDA(cudaMemcpyAsync(data + (size_t)n * nin, T, (size_t)n * nout * sizeof(float), cudaMemcpyDefault,
                                  c.stream));
        SAGB_CUDA(cudaMemcpyAsync(data + (size_t)n * (nin + nout), M, (size_t)n * nout * sizeof(float),
                                  cudaMemcpyDefault, c.stream));
    }
    loaded_n = n;
}

void Mlp::gather(Ctx &c, const int *perm, int off, int B, bool targets) {
    const int n = loaded_n;
    const float *X = data, *T = targets ? data + (size_t)n * nin : nullptr,
                *M = targets ? data + (size_t)n * (nin + nout) : nullptr;
    float *Xb = ws, *Y = Xb + (size_t)ws_batch * (nin + 2 * hid), *Tb = Y + (size_t)ws_batch * nout,
          *Mb = Tb + (size_t)ws_batch * nout;
    const int tot = B * (nin + nout);
    k_gather_norm<<<(tot + 255) / 256, 256, 0, c.stream>>>(X, T, M, perm, off, B, nin, nout, norm, norm + nin, Xb,
                                                          Tb, Mb);
    c.launches++;
}

void Mlp::predict(Ctx &c, const float *X, int n, float *Y) {
    reserve(n);
    load(c, X, nullptr, nullptr, n);
    gather(c, nullptr, 0, n, false);
    forward_batch(c, n);
    const float *Yd = ws + (size_t)ws_batch * (nin + 2 * hid);
    SAGB_CUDA(cudaMemcpyAsync(Y, Yd, (size_t)n * nout * sizeof(float), cudaMemcpyDefault, c.stream));
    SAGB_CUDA(cudaStreamSynchronize(c.stream));
}

float Mlp::gradient(Ctx &c, const float *X, const float *T, const float *M, int n, float *grad) {
    reserve(n);
    load(c, X, T, M, n);
    gather(c, nullptr, 0, n, true);
    forward_batch(c, n);
    backward_batch(c, n);
    float loss = 0.f;
    SAGB_CUDA(cudaMemcpyAsync(&loss, loss_slot(), sizeof(float), cudaMemcpyDeviceToHost, c.stream));
    if (grad)
        SAGB_CUDA(cudaMemcpyAsync(grad, g, nparams() * sizeof(float), cudaMemcpyDefault, c.stream));
    SAGB_CUDA(cudaStreamSynchronize(c.stream));
    return loss;
}

void Mlp::train(Ctx &c, const float *X, const float *T, const float *M, int n, int epochs, int batch, float lr,
                uint64_t seed, float *loss_hist) {
    if (n < 1 || epochs < 1 || batch < 1) throw CudaError{"invalid training arguments"};
    batch = std::min(batch, n);
    reserve(batch);
    load(c, X, T, M, n);
    dfree(perm_d);
    perm_d = (int *)dmalloc((size_t)n * sizeof(int));
    std::vector<int> perm(n);
    std::vector<float> ep_loss((size_t)epochs, 0.f);
    const int steps_per_epoch = (n + batch - 1) / batch;
    float *dloss = (float *)dmalloc((size_t)epochs * steps_per_epoch * sizeof(float));
    uint64_t st = seed;
    auto next = [&]() {
        uint64_t z = (st += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    const int np = (int)nparams();
    const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    for (int e = 0; e < epochs; e++) {
        for (int i = 0; i < n; i++) perm[i] = i;
        for (int i = n - 1; i > 0; i--) std::swap(perm[i], perm[next() % (uint64_t)(i + 1)]);  // Fisher-Yates
        SAGB_CUDA(cudaMemcpyAsync(perm_d, perm.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, c.stream));
        SAGB_CUDA(cudaStreamSynchronize(c.stream));  // perm is reused next epoch
        for (int s = 0; s < steps_per_epoch; s++) {
            const int off = s * batch, B = std::min(batch, n - off);
            gather(c, perm_d, off, B, true);
            forward_batch(c, B);
            backward_batch(c, B);
            SAGB_CUDA(cudaMemcpyAsync(dloss + (size_t)e * steps_per_epoch + s, loss_slot(), sizeof(float),
                                      cudaMemcpyDeviceToDevice, c.stream));
            t++;
            const float bc1 = 1.f - std::pow(beta1, (float)t), bc2 = 1.f - std::pow(beta2, (float)t);
            k_adam<<<(np + 255) / 256, 256, 0, c.stream>>>(p, g, m1, m2, np, lr, beta1, beta2, eps, bc1, bc2);
            c.launches++;
        }
    }
    std::vector<float> all((size_t)epochs * steps_per_epoch);
    SAGB_CUDA(cudaMemcpyAsync(all.data(), dloss, all.size() * sizeof(float), cudaMemcpyDeviceToHost, c.stream));
    SAGB_CUDA(cudaStreamSynchronize(c.stream));
    dfree(dloss);
    if (loss_hist)
        for (int e = 0; e < epochs; e++) {
            float s = 0.f;
            for (int k = 0; k < steps_per_epoch; k++) s += all[(size_t)e * steps_per_epoch + k];
            loss_hist[e] = s / steps_per_epoch;
        }
}

void Mlp::get_params(float *out) const {
    SAGB_CUDA(cudaMemcpy(out, p, nparams() * sizeof(float), cudaMemcpyDeviceToHost));
}

void Mlp::set_params(const float *in) {
    SAGB_CUDA(cudaMemcpy(p, in, nparams() * sizeof(float), cudaMemcpyHostToDevice));
    SAGB_CUDA(cudaMemset(m1, 0, 2 * nparams() * sizeof(float)));
    t = 0;
}

}  // namespace sagb
