// rp_mlp.cu -- the band-tail MLP: training and inference kernels (K8).
//
// A small fully connected network (nin -> nhid -> nhid -> nout, ReLU between
// the layers) predicts the part of chi0 that the bands above a truncation add,
// per |q+G| shell, from features of the truncated-band chi0 and the band
// energies (respackdev_gb300/tail.py builds the features and applies the
// correction).  The reference has no counterpart: the full band sum is both the
// training target and the measure of the network's error.
//
// Weights live as an FP32 master copy (Adam updates it) and a BF16 copy that
// the forward and backward passes read; every product accumulates in FP32.
// Parameter layout (also the host-visible order): W1 [nhid][nin], b1 [nhid],
// W2 [nhid][nhid], b2 [nhid], W3 [nout][nhid], b3 [nout].
// Loss: mean squared error over the batch and the outputs.
#include <cuda_bf16.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "rp_dev.cuh"
#include "rp_host.h"

struct rp_mlp {
  int nin = 0, nhid = 0, nout = 0, dev = 0;
  size_t np = 0;                     // parameter count
  size_t oW1, ob1, oW2, ob2, oW3, ob3;
  float *p = nullptr, *g = nullptr, *m1 = nullptr, *m2 = nullptr;  // master, gradient, Adam moments
  __nv_bfloat16 *pb = nullptr;       // BF16 copy used by the passes
  float *act = nullptr;              // per-batch activations and their gradients
  size_t act_cap = 0;                // samples the activation buffers hold
  float *io = nullptr;               // x, t, y staging
  size_t io_cap = 0;
  float *loss = nullptr;             // device scalar
  long long step = 0;
  cudaStream_t st = nullptr;
  std::string err;
};

namespace rp {

// Y[b][j] = act(sum_i X[b][i] W[j][i] + c[j]); pre-activation kept in Z when relu
__global__ void mlp_dense_fwd(const float *__restrict__ X, int B, int K, const __nv_bfloat16 *__restrict__ W,
                              const __nv_bfloat16 *__restrict__ c, int N, int relu, float *__restrict__ Z,
                              float *__restrict__ Y) {
  extern __shared__ float xs[];  // 32 samples x K
  const int b0 = blockIdx.x * 32;
  for (int l = threadIdx.x; l < 32 * K; l += blockDim.x) {
    const int bb = l / K, i = l % K;
    xs[l] = b0 + bb < B ? X[(size_t)(b0 + bb) * K + i] : 0.f;
  }
  __syncthreads();
  for (int o = threadIdx.x; o < 32 * N; o += blockDim.x) {
    const int bb = o / N, j = o % N;
    if (b0 + bb >= B) continue;
    float s = __bfloat162float(c[j]);
    const __nv_bfloat16 *w = W + (size_t)j * K;
    const float *x = xs + (size_t)bb * K;
    for (int i = 0; i < K; i++) s = fmaf(x[i], __bfloat162float(w[i]), s);
    if (relu) {
      Z[(size_t)(b0 + bb) * N + j] = s;
      s = fmaxf(s, 0.f);
    }
    Y[(size_t)(b0 + bb) * N + j] = s;
  }
}

// dX[b][i] = sum_j dY[b][j] W[j][i] (then times the ReLU mask of the layer below)
__global__ void mlp_dense_bwd_x(const float *__restrict__ dY, int B, int N, const __nv_bfloat16 *__restrict__ W, int K,
                                const float *__restrict__ Zbelow, float *__restrict__ dX) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)B * K) return;
  const int b = (int)(idx / K), i = (int)(idx % K);
  float s = 0.f;
  for (int j = 0; j < N; j++) s = fmaf(dY[(size_t)b * N + j], __bfloat162float(W[(size_t)j * K + i]), s);
  if (Zbelow && !(Zbelow[idx] > 0.f)) s = 0.f;
  dX[idx] = s;
}

// dW[j][i] += sum_b dY[b][j] X[b][i], dc[j] += sum_b dY[b][j]
__global__ void mlp_dense_bwd_w(const float *__restrict__ dY, const float *__restrict__ X, int B, int N, int K,
                                float *__restrict__ dW, float *__restrict__ dc) {
  const int j = blockIdx.x;
  for (int i = threadIdx.x; i <= K; i += blockDim.x) {
    float s = 0.f;
    if (i < K)
      for (int b = 0; b < B; b++) s = fmaf(dY[(size_t)b * N + j], X[(size_t)b * K + i], s);
    else
      for (int b = 0; b < B; b++) s += dY[(size_t)b * N + j];
    if (i < K) dW[(size_t)j * K + i] += s;
    else dc[j] += s;
  }
}

// dY = 2 (Y - T) / (B nout); loss += sum (Y - T)^2 / (B nout)
__global__ void mlp_mse(const float *__restrict__ Y, const float *__restrict__ T, size_t n, float inv,
                        float *__restrict__ dY, float *__restrict__ loss) {
  float acc = 0.f;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float d = Y[i] - T[i];
    dY[i] = 2.f * d * inv;
    acc = fmaf(d * inv, d, acc);
  }
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc);
}

__global__ void mlp_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m1,
                         float *__restrict__ m2, size_t n, float lr, float b1, float b2, float eps, float c1, float c2,
                         __nv_bfloat16 *__restrict__ pb) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float a = b1 * m1[i] + (1.f - b1) * gi, v = b2 * m2[i] + (1.f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = v;
    const float q = p[i] - lr * (a * c1) / (sqrtf(v * c2) + eps);
    p[i] = q;
    pb[i] = __float2bfloat16_rn(q);
  }
}

__global__ void mlp_to_bf16(const float *__restrict__ p, size_t n, __nv_bfloat16 *__restrict__ pb) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    pb[i] = __float2bfloat16_rn(p[i]);
}

}  // namespace rp

namespace {

using rp::fail;

void ensure_act(rp_mlp *m, int B) {
  if ((size_t)B <= m->act_cap) return;
  if (m->act) cudaFree(m->act);
  // Z1, H1, Z2, H2, Y, dY, dH2, dH1
  const size_t per = 4 * (size_t)m->nhid + 2 * (size_t)m->nout + 2 * (size_t)m->nhid;
  RP_CUDA(cudaMalloc(&m->act, sizeof(float) * per * (size_t)B));
  m->act_cap = (size_t)B;
}
void ensure_io(rp_mlp *m, int B) {
  if ((size_t)B <= m->io_cap) return;
  if (m->io) cudaFree(m->io);
  RP_CUDA(cudaMalloc(&m->io, sizeof(float) * (size_t)B * (m->nin + 2 * m->nout)));
  m->io_cap = (size_t)B;
}

struct Act {
  float *Z1, *H1, *Z2, *H2, *Y, *dY, *dH2, *dH1;
};
Act acts(rp_mlp *m, int B) {
  Act a;
  const size_t h = (size_t)m->nhid * B, o = (size_t)m->nout * B;
  a.Z1 = m->act; a.H1 = a.Z1 + h; a.Z2 = a.H1 + h; a.H2 = a.Z2 + h;
  a.Y = a.H2 + h; a.dY = a.Y + o; a.dH2 = a.dY + o; a.dH1 = a.dH2 + h;
  return a;
}

// forward on device inputs X (B x nin) on stream st (default: the network's
// own); leaves the activations in m->act
void forward(rp_mlp *m, const float *X, int B, cudaStream_t st = nullptr) {
  if (!st) st = m->st;
  ensure_act(m, B);
  Act a = acts(m, B);
  const unsigned nb = (unsigned)((B + 31) / 32);
  const __nv_bfloat16 *pb = m->pb;
  rp::mlp_dense_fwd<<<nb, 256, sizeof(float) * 32 * m->nin, st>>>(X, B, m->nin, pb + m->oW1, pb + m->ob1, m->nhid, 1,
                                                                  a.Z1, a.H1);
  rp::mlp_dense_fwd<<<nb, 256, sizeof(float) * 32 * m->nhid, st>>>(a.H1, B, m->nhid, pb + m->oW2, pb + m->ob2,
                                                                   m->nhid, 1, a.Z2, a.H2);
  rp::mlp_dense_fwd<<<nb, 256, sizeof(float) * 32 * m->nhid, st>>>(a.H2, B, m->nhid, pb + m->oW3, pb + m->ob3,
                                                                   m->nout, 0, nullptr, a.Y);
  RP_CUDA(cudaGetLastError());
}

// loss and gradients (into m->g, cleared first) for device inputs X, targets T
void backward(rp_mlp *m, const float *X, const float *T, int B) {
  Act a = acts(m, B);
  const __nv_bfloat16 *pb = m->pb;
  RP_CUDA(cudaMemsetAsync(m->g, 0, sizeof(float) * m->np, m->st));
  RP_CUDA(cudaMemsetAsync(m->loss, 0, sizeof(float), m->st));
  const size_t no = (size_t)B * m->nout, nh = (size_t)B * m->nhid;
  rp::mlp_mse<<<(unsigned)std::min<size_t>((no + 255) / 256, 1024), 256, 0, m->st>>>(a.Y, T, no,
                                                                                     1.f / (float)no, a.dY, m->loss);
  // layer 3
  rp::mlp_dense_bwd_w<<<m->nout, 128, 0, m->st>>>(a.dY, a.H2, B, m->nout, m->nhid, m->g + m->oW3, m->g + m->ob3);
  rp::mlp_dense_bwd_x<<<(unsigned)((nh + 255) / 256), 256, 0, m->st>>>(a.dY, B, m->nout, pb + m->oW3, m->nhid, a.Z2,
                                                                       a.dH2);
  // layer 2
  rp::mlp_dense_bwd_w<<<m->nhid, 128, 0, m->st>>>(a.dH2, a.H1, B, m->nhid, m->nhid, m->g + m->oW2, m->g + m->ob2);
  rp::mlp_dense_bwd_x<<<(unsigned)((nh + 255) / 256), 256, 0, m->st>>>(a.dH2, B, m->nhid, pb + m->oW2, m->nhid, a.Z1,
                                                                       a.dH1);
  // layer 1
  rp::mlp_dense_bwd_w<<<m->nhid, 128, 0, m->st>>>(a.dH1, X, B, m->nhid, m->nin, m->g + m->oW1, m->g + m->ob1);
  RP_CUDA(cudaGetLastError());
}

}  // namespace

const float *rp::mlp_forward_device(rp_mlp *m, const float *X, int B, cudaStream_t st) {
  // the network's own stream may still be finishing a set_params upload
  RP_CUDA(cudaStreamSynchronize(m->st));
  forward(m, X, B, st);
  return acts(m, B).Y;
}

namespace {

template <typename F>
int guarded(rp_mlp *m, F &&f) {
  try {
    if (m) RP_CUDA(cudaSetDevice(m->dev));
    f();
    return 0;
  } catch (const rp::Error &e) {
    if (m) m->err = e.what();
    rp::set_global_error(e.what());
    return e.code;
  }
}

}  // namespace

extern "C" {

int rp_mlp_create(rp_mlp **out, int nin, int nhid, int nout, unsigned long long seed, int device) {
  if (!out) return 1;
  *out = nullptr;
  rp_mlp *m = new rp_mlp;
  m->dev = device;
  const int rc = guarded(m, [&] {
    // a forward block stages 32 samples x max(nin, nhid) floats in shared memory
    if (nin < 1 || nhid < 1 || nout < 1 || nin > 256 || nhid > 256 || nout > 256)
      fail(1, "MLP sizes must be in 1..256 (got %d, %d, %d)", nin, nhid, nout);
    m->nin = nin; m->nhid = nhid; m->nout = nout;
    m->oW1 = 0; m->ob1 = m->oW1 + (size_t)nhid * nin;
    m->oW2 = m->ob1 + nhid; m->ob2 = m->oW2 + (size_t)nhid * nhid;
    m->oW3 = m->ob2 + nhid; m->ob3 = m->oW3 + (size_t)nout * nhid;
    m->np = m->ob3 + nout;
    RP_CUDA(cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking));
    RP_CUDA(cudaMalloc(&m->p, sizeof(float) * m->np * 4));
    m->g = m->p + m->np; m->m1 = m->g + m->np; m->m2 = m->m1 + m->np;
    RP_CUDA(cudaMalloc(&m->pb, sizeof(__nv_bfloat16) * m->np));
    RP_CUDA(cudaMalloc(&m->loss, sizeof(float)));
    // He-uniform initial weights from a 64-bit LCG, zero biases
    std::vector<float> h(m->np, 0.f);
    unsigned long long s = seed * 6364136223846793005ULL + 1442695040888963407ULL;
    auto uni = [&]() {
      s = s * 6364136223846793005ULL + 1442695040888963407ULL;
      return (float)((s >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f;
    };
    auto fill = [&](size_t o, int rows, int cols) {
      const float lim = std::sqrt(6.f / (float)cols);
      for (size_t i = 0; i < (size_t)rows * cols; i++) h[o + i] = lim * uni();
    };
    fill(m->oW1, nhid, nin);
    fill(m->oW2, nhid, nhid);
    fill(m->oW3, nout, nhid);
    RP_CUDA(cudaMemcpyAsync(m->p, h.data(), sizeof(float) * m->np, cudaMemcpyHostToDevice, m->st));
    RP_CUDA(cudaMemsetAsync(m->m1, 0, sizeof(float) * m->np * 2, m->st));
    rp::mlp_to_bf16<<<256, 256, 0, m->st>>>(m->p, m->np, m->pb);
    RP_CUDA(cudaStreamSynchronize(m->st));
  });
  if (rc) { rp_mlp_destroy(m); return rc; }
  *out = m;
  return 0;
}

int rp_mlp_nparams(const rp_mlp *m) { return m ? (int)m->np : 0; }

int rp_mlp_get_params(rp_mlp *m, float *params) {
  if (!m || !params) return 1;
  return guarded(m, [&] {
    RP_CUDA(cudaMemcpyAsync(params, m->p, sizeof(float) * m->np, cudaMemcpyDeviceToHost, m->st));
    RP_CUDA(cudaStreamSynchronize(m->st));
  });
}

int rp_mlp_set_params(rp_mlp *m, const float *params) {
  if (!m || !params) return 1;
  return guarded(m, [&] {
    RP_CUDA(cudaMemcpyAsync(m->p, params, sizeof(float) * m->np, cudaMemcpyHostToDevice, m->st));
    RP_CUDA(cudaMemsetAsync(m->m1, 0, sizeof(float) * m->np * 2, m->st));
    m->step = 0;
    rp::mlp_to_bf16<<<256, 256, 0, m->st>>>(m->p, m->np, m->pb);
    RP_CUDA(cudaStreamSynchronize(m->st));
  });
}

int rp_mlp_forward(rp_mlp *m, const float *x, int B, float *y) {
  if (!m || !x || !y || B < 1) return 1;
  return guarded(m, [&] {
    ensure_io(m, B);
    float *X = m->io;
    RP_CUDA(cudaMemcpyAsync(X, x, sizeof(float) * (size_t)B * m->nin, cudaMemcpyHostToDevice, m->st));
    forward(m, X, B);
    RP_CUDA(cudaMemcpyAsync(y, acts(m, B).Y, sizeof(float) * (size_t)B * m->nout, cudaMemcpyDeviceToHost, m->st));
    RP_CUDA(cudaStreamSynchronize(m->st));
  });
}

int rp_mlp_gradients(rp_mlp *m, const float *x, const float *t, int B, float *loss, float *grad) {
  if (!m || !x || !t || B < 1) return 1;
  return guarded(m, [&] {
    ensure_io(m, B);
    float *X = m->io, *T = X + (size_t)B * m->nin;
    RP_CUDA(cudaMemcpyAsync(X, x, sizeof(float) * (size_t)B * m->nin, cudaMemcpyHostToDevice, m->st));
    RP_CUDA(cudaMemcpyAsync(T, t, sizeof(float) * (size_t)B * m->nout, cudaMemcpyHostToDevice, m->st));
    forward(m, X, B);
    backward(m, X, T, B);
    if (loss) RP_CUDA(cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->st));
    if (grad) RP_CUDA(cudaMemcpyAsync(grad, m->g, sizeof(float) * m->np, cudaMemcpyDeviceToHost, m->st));
    RP_CUDA(cudaStreamSynchronize(m->st));
  });
}

// `steps` Adam steps over the n samples in minibatches of `batch`, taken in a
// fixed order (sample i of step s is (s * batch + i) mod n); losses[s] = the
// minibatch loss before step s.
int rp_mlp_train(rp_mlp *m, const float *x, const float *t, int n, int steps, int batch, float lr, float *losses) {
  if (!m || !x || !t || n < 1 || steps < 0 || batch < 1) return 1;
  return guarded(m, [&] {
    const int B = std::min(batch, n);
    ensure_io(m, n);
    float *X = m->io, *T = X + (size_t)n * m->nin;
    RP_CUDA(cudaMemcpyAsync(X, x, sizeof(float) * (size_t)n * m->nin, cudaMemcpyHostToDevice, m->st));
    RP_CUDA(cudaMemcpyAsync(T, t, sizeof(float) * (size_t)n * m->nout, cudaMemcpyHostToDevice, m->st));
    float *xb = nullptr;
    RP_CUDA(cudaMalloc(&xb, sizeof(float) * (size_t)B * (m->nin + m->nout)));
    float *tb = xb + (size_t)B * m->nin;
    std::vector<float> lh(steps);
    for (int s = 0; s < steps; s++) {
      // gather the minibatch (contiguous runs, wrapping at n)
      int off = (int)(((long long)s * B) % n), got = 0;
      while (got < B) {
        const int take = std::min(B - got, n - off);
        RP_CUDA(cudaMemcpyAsync(xb + (size_t)got * m->nin, X + (size_t)off * m->nin, sizeof(float) * take * m->nin,
                                cudaMemcpyDeviceToDevice, m->st));
        RP_CUDA(cudaMemcpyAsync(tb + (size_t)got * m->nout, T + (size_t)off * m->nout,
                                sizeof(float) * take * m->nout, cudaMemcpyDeviceToDevice, m->st));
        got += take;
        off = 0;
      }
      forward(m, xb, B);
      backward(m, xb, tb, B);
      RP_CUDA(cudaMemcpyAsync(&lh[s], m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->st));
      m->step++;
      const float b1 = 0.9f, b2 = 0.999f;
      const float c1 = 1.f / (1.f - std::pow(b1, (float)m->step)), c2 = 1.f / (1.f - std::pow(b2, (float)m->step));
      rp::mlp_adam<<<256, 256, 0, m->st>>>(m->p, m->g, m->m1, m->m2, m->np, lr, b1, b2, 1e-8f, c1, c2, m->pb);
    }
    RP_CUDA(cudaGetLastError());
    RP_CUDA(cudaStreamSynchronize(m->st));
    cudaFree(xb);
    if (losses) std::memcpy(losses, lh.data(), sizeof(float) * steps);
  });
}

const char *rp_mlp_last_error(const rp_mlp *m) { return m ? m->err.c_str() : ""; }

void rp_mlp_destroy(rp_mlp *m) {
  if (!m) return;
  cudaSetDevice(m->dev);
  if (m->p) cudaFree(m->p);
  if (m->pb) cudaFree(m->pb);
  if (m->act) cudaFree(m->act);
  if (m->io) cudaFree(m->io);
  if (m->loss) cudaFree(m->loss);
  if (m->st) cudaStreamDestroy(m->st);
  delete m;
}

}  // extern "C"
