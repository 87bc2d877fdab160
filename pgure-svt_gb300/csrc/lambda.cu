// lambda.cu — learned lambda proposal (not in the reference).
//
// A small MLP maps per-window features (the risk's noise parameters and a
// histogram of log singular values) to y = log10(lambda/upper); the proposal
// starts a narrow PGURE search (eval.cu, phase 1) that falls back to the plain
// search.  The network is tiny (67 -> 128 -> 128 -> 128 -> 1, 41,857
// parameters), so every pass is one CUDA-core kernel over blocks of 32
// samples: weights are read as bf16 from global memory (they stay in L1),
// activations live in shared memory, sums are FP32.  Training keeps FP32
// master weights and a bf16 shadow that the passes read; per-block gradient
// partials are summed in a fixed order, so training is deterministic.
#include <cuda_bf16.h>

#include "pgsvt.h"
#include "pgsvt_internal.h"

namespace pgsvt {
namespace lam {

constexpr int NF = PGSVT_LAMBDA_FEATURES;   // 67
constexpr int H = PGSVT_LAMBDA_HIDDEN;      // 128
constexpr int SB = 32;                      // samples per block
constexpr int LD0 = NF + 2;                 // 69: odd row strides keep the
constexpr int LDH = H + 1;                  // column reads conflict-free
constexpr int OFF_MEAN = 0, OFF_SCALE = NF, OFF_W1 = 2 * NF;
constexpr int OFF_B1 = OFF_W1 + H * NF, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + H * H;
constexpr int OFF_W3 = OFF_B2 + H, OFF_B3 = OFF_W3 + H * H, OFF_W4 = OFF_B3 + H;
constexpr int OFF_B4 = OFF_W4 + H, OFF_YMEAN = OFF_B4 + 1, OFF_YSCALE = OFF_YMEAN + 1;
constexpr int TOTAL = OFF_YSCALE + 1;
constexpr int NPARAM = OFF_YMEAN - OFF_W1;
static_assert(TOTAL == PGSVT_LAMBDA_MODEL_FLOATS, "model layout");
static_assert(NPARAM == PGSVT_LAMBDA_PARAMS, "parameter count");
static_assert(OFF_W1 == PGSVT_LAMBDA_PARAM_OFFSET, "parameter offset");

struct Smem {
  float x0[SB * LD0];
  float z[3][SB * LDH];   // pre-activations, then their gradients
  float a[3][SB * LDH];   // activations
  float o[SB];            // network outputs (before y_scale / y_mean)
  float dO[SB];
  float red[4];
};

__device__ __forceinline__ float gelu(float z) {
  return 0.5f * z * (1.f + erff(z * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_grad(float z) {
  return 0.5f * (1.f + erff(z * 0.70710678118654752f)) +
         z * 0.39894228040143268f * expf(-0.5f * z * z);
}
__device__ __forceinline__ float wb(const __nv_bfloat16* W, int i) {
  return __bfloat162float(W[i]);
}

// One dense layer plus GELU: thread j computes output j for every sample.
template <int KIN>
__device__ void dense_gelu(const __nv_bfloat16* W, const float* b, const float* in, int ld_in,
                           float* z, float* a) {
  const int j = threadIdx.x;
  float acc[SB];
  const float bj = b[j];
#pragma unroll
  for (int s = 0; s < SB; ++s) acc[s] = bj;
  for (int k = 0; k < KIN; ++k) {
    const float w = wb(W, j * KIN + k);
#pragma unroll
    for (int s = 0; s < SB; ++s) acc[s] = fmaf(w, in[s * ld_in + k], acc[s]);
  }
#pragma unroll
  for (int s = 0; s < SB; ++s) {
    z[s * LDH + j] = acc[s];
    a[s * LDH + j] = gelu(acc[s]);
  }
}

// Forward pass of samples [0, ns) held in sm.x0 (already normalised); the
// outputs land in sm.o.  128 threads.
__device__ void forward(const float* m, const __nv_bfloat16* wbf, Smem& sm) {
  dense_gelu<NF>(wbf + OFF_W1, m + OFF_B1, sm.x0, LD0, sm.z[0], sm.a[0]);
  __syncthreads();
  dense_gelu<H>(wbf + OFF_W2, m + OFF_B2, sm.a[0], LDH, sm.z[1], sm.a[1]);
  __syncthreads();
  dense_gelu<H>(wbf + OFF_W3, m + OFF_B3, sm.a[1], LDH, sm.z[2], sm.a[2]);
  __syncthreads();
  if (threadIdx.x < SB) {
    const int s = threadIdx.x;
    float acc = m[OFF_B4];
    for (int k = 0; k < H; ++k) acc = fmaf(wb(wbf, OFF_W4 + k), sm.a[2][s * LDH + k], acc);
    sm.o[s] = acc;
  }
  __syncthreads();
}

// Stage features rows [r0, r0+ns) into sm.x0 as (f - mean) * scale, rows
// beyond ns as zeros.  `rows` maps a block row to a feature row (or null).
__device__ void load_inputs(const float* m, const float* feat, const int32_t* rows, int r0,
                            int ns, Smem& sm) {
  for (int i = threadIdx.x; i < SB * NF; i += blockDim.x) {
    const int s = i / NF, k = i % NF;
    float v = 0.f;
    if (s < ns) {
      const int r = rows ? rows[r0 + s] : r0 + s;
      v = (feat[(size_t)r * NF + k] - m[OFF_MEAN + k]) * m[OFF_SCALE + k];
    }
    sm.x0[s * LD0 + k] = v;
  }
  __syncthreads();
}

// Weight gradients of one layer (thread k owns input column k) and the
// gradient of its input, through GELU when `zprev` is given.
template <int KIN>
__device__ void dense_backward(const __nv_bfloat16* W, const float* dz, const float* in,
                               int ld_in, float* gW, float* gb, float* zprev) {
  const int k = threadIdx.x;
  float acol[SB];
#pragma unroll
  for (int s = 0; s < SB; ++s) acol[s] = (k < KIN) ? in[s * ld_in + k] : 0.f;
  float din[SB];
#pragma unroll
  for (int s = 0; s < SB; ++s) din[s] = 0.f;
  for (int j = 0; j < H; ++j) {
    float g = 0.f;
    const float w = (k < KIN) ? wb(W, j * KIN + k) : 0.f;
#pragma unroll
    for (int s = 0; s < SB; ++s) {
      const float d = dz[s * LDH + j];
      g = fmaf(d, acol[s], g);
      din[s] = fmaf(w, d, din[s]);
    }
    if (k < KIN) gW[j * KIN + k] = g;
  }
  {
    const int j = threadIdx.x;  // H threads: bias gradient of output j
    float g = 0.f;
#pragma unroll
    for (int s = 0; s < SB; ++s) g += dz[s * LDH + j];
    gb[j] = g;
  }
  __syncthreads();  // every read of dz and of the previous z is done
  if (zprev && k < KIN) {
#pragma unroll
    for (int s = 0; s < SB; ++s) zprev[s * LDH + k] = din[s] * gelu_grad(zprev[s * LDH + k]);
  }
  __syncthreads();
}

// Forward + backward of one block of samples; writes the block's gradient
// partial (NPARAM floats, already divided by `norm`) and its squared-error sum.
__global__ void __launch_bounds__(H) k_mlp_grad(const float* __restrict__ m,
                                                const __nv_bfloat16* __restrict__ wbf,
                                                const float* __restrict__ feat,
                                                const float* __restrict__ target,
                                                const int32_t* __restrict__ perm,
                                                const int* __restrict__ epoch, int64_t perm_stride,
                                                int r0, int n, float norm, float* __restrict__ part,
                                                float* __restrict__ part_loss) {
  extern __shared__ float smraw[];
  Smem& sm = *reinterpret_cast<Smem*>(smraw);
  const int b0 = r0 + blockIdx.x * SB;
  const int ns = max(0, min(SB, n - b0));
  const int32_t* rows = perm ? perm + (epoch ? (int64_t)(*epoch) * perm_stride : 0) : nullptr;
  load_inputs(m, feat, rows, b0, ns, sm);
  forward(m, wbf, sm);
  const float ym = m[OFF_YMEAN], ysi = 1.f / m[OFF_YSCALE];
  if (threadIdx.x < SB) {
    const int s = threadIdx.x;
    float e = 0.f;
    if (s < ns) {
      const int r = rows ? rows[b0 + s] : b0 + s;
      e = sm.o[s] - (target[r] - ym) * ysi;
    }
    sm.dO[s] = 2.f * e * norm;
    float sq = e * e;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
    if (s == 0) part_loss[blockIdx.x] = sq;
  }
  __syncthreads();
  float* g = part + (size_t)blockIdx.x * NPARAM;
  // output layer: dW4[k] = sum_s dO a3, da3 = dO W4, dz3 = da3 gelu'(z3)
  {
    const int k = threadIdx.x;
    float gw = 0.f, gbias = 0.f;
    const float w4 = wb(wbf, OFF_W4 + k);
#pragma unroll
    for (int s = 0; s < SB; ++s) {
      gw = fmaf(sm.dO[s], sm.a[2][s * LDH + k], gw);
      gbias += sm.dO[s];
    }
    g[OFF_W4 - OFF_W1 + k] = gw;
    if (k == 0) g[OFF_B4 - OFF_W1] = gbias;
    __syncthreads();
#pragma unroll
    for (int s = 0; s < SB; ++s)
      sm.z[2][s * LDH + k] = sm.dO[s] * w4 * gelu_grad(sm.z[2][s * LDH + k]);
    __syncthreads();
  }
  dense_backward<H>(wbf + OFF_W3, sm.z[2], sm.a[1], LDH, g + (OFF_W3 - OFF_W1),
                    g + (OFF_B3 - OFF_W1), sm.z[1]);
  dense_backward<H>(wbf + OFF_W2, sm.z[1], sm.a[0], LDH, g + (OFF_W2 - OFF_W1),
                    g + (OFF_B2 - OFF_W1), sm.z[0]);
  dense_backward<NF>(wbf + OFF_W1, sm.z[0], sm.x0, LD0, g + 0, g + (OFF_B1 - OFF_W1), nullptr);
}

// Network outputs y (after y_scale / y_mean) of n feature rows.
__global__ void __launch_bounds__(H) k_mlp_forward(const float* __restrict__ m,
                                                   const __nv_bfloat16* __restrict__ wbf,
                                                   const float* __restrict__ feat, int n,
                                                   float* __restrict__ y) {
  extern __shared__ float smraw[];
  Smem& sm = *reinterpret_cast<Smem*>(smraw);
  const int b0 = blockIdx.x * SB;
  const int ns = max(0, min(SB, n - b0));
  load_inputs(m, feat, nullptr, b0, ns, sm);
  forward(m, wbf, sm);
  if (threadIdx.x < ns) y[b0 + threadIdx.x] = sm.o[threadIdx.x] * m[OFF_YSCALE] + m[OFF_YMEAN];
}

__device__ __forceinline__ bool is_weight(int i) {  // i: offset in the model
  return (i >= OFF_W1 && i < OFF_B1) || (i >= OFF_W2 && i < OFF_B2) ||
         (i >= OFF_W3 && i < OFF_B3) || (i >= OFF_W4 && i < OFF_B4);
}

// bf16 shadow of the whole model (only the weight ranges are read as bf16).
__global__ void k_mlp_shadow(const float* __restrict__ m, __nv_bfloat16* __restrict__ wbf) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < TOTAL; i += gridDim.x * blockDim.x)
    wbf[i] = __float2bfloat16_rn(m[i]);
}

// Sum of the block partials in block order (gradient entry point).
__global__ void k_mlp_gsum(const float* __restrict__ part, int nblk, float* __restrict__ grad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NPARAM) return;
  float g = 0.f;
  for (int b = 0; b < nblk; ++b) g += part[(size_t)b * NPARAM + i];
  grad[i] = g;
}

struct AdamCfg {
  float lr, lr_final, wd, b1, b2, eps;
  int steps_per_epoch, total_steps;
};

// AdamW step `step` of the epoch in *epoch: gradient = sum of the block
// partials in block order; FP32 master and moments, bf16 shadow refreshed.
__global__ void k_mlp_adam(float* __restrict__ m, __nv_bfloat16* __restrict__ wbf,
                           float* __restrict__ mom1, float* __restrict__ mom2,
                           const float* __restrict__ part, int nblk,
                           const int* __restrict__ epoch, int step, AdamCfg c) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NPARAM) return;
  const int t = *epoch * c.steps_per_epoch + step + 1;  // 1-based step count
  const float prog = (float)(t - 1) / (float)max(1, c.total_steps - 1);
  const float lr = c.lr_final + 0.5f * (c.lr - c.lr_final) * (1.f + cospif(prog));
  float g = 0.f;
  for (int b = 0; b < nblk; ++b) g += part[(size_t)b * NPARAM + i];
  const float m1 = c.b1 * mom1[i] + (1.f - c.b1) * g;
  const float m2 = c.b2 * mom2[i] + (1.f - c.b2) * g * g;
  mom1[i] = m1;
  mom2[i] = m2;
  const float bc1 = 1.f - powf(c.b1, (float)t), bc2 = 1.f - powf(c.b2, (float)t);
  const int mi = OFF_W1 + i;
  float w = m[mi];
  if (is_weight(mi)) w -= lr * c.wd * w;
  w -= lr * (m1 / bc1) / (sqrtf(m2 / bc2) + c.eps);
  m[mi] = w;
  wbf[mi] = __float2bfloat16_rn(w);
}

// Mean loss of the epoch; advances the device epoch counter.
__global__ void k_mlp_epoch_end(const float* __restrict__ loss_acc, int nsteps, int nblk, int n,
                                int* __restrict__ epoch, float* __restrict__ epoch_loss) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  float t = 0.f;
  for (int i = 0; i < nsteps * nblk; ++i) t += loss_acc[i];
  epoch_loss[*epoch] = t / (float)max(1, n);
  *epoch += 1;
}

}  // namespace lam

// ---------------------------------------------------------------------------
// Features of every window of a batch: block w histograms the copy-0
// singular values of the sampled patches of window w.
__global__ void __launch_bounds__(256) k_lambda_features(Problem pb, DeviceBuffers d) {
  const Geometry& g = pb.g;
  const int w = blockIdx.x;
  __shared__ int hist[64];
  if (threadIdx.x < 64) hist[threadIdx.x] = 0;
  __syncthreads();
  const int ns = d.nfeat_slots, nwin = g.nwin;
  const size_t NP = g.NP;
  const float* sv = d.sv + (size_t)w * 4 * g.NC * NP;  // copy 0
  for (int i = threadIdx.x; i < ns * nwin; i += blockDim.x) {
    const int si = i / nwin, t = i % nwin;
    const float s = sv[(size_t)t * NP + d.feat_slots[si]];
    int b = 0;
    if (s > 0.f && isfinite(s)) {
      const float x = (log10f(s) + 4.f) * (64.f / 6.f);
      b = x <= 0.f ? 0 : (x >= 63.f ? 63 : (int)x);
    }
    atomicAdd(&hist[b], 1);
  }
  __syncthreads();
  float* f = d.feat + (size_t)w * lam::NF;
  const WinConst& wc = d.wc[w];
  if (threadIdx.x < 64) f[3 + threadIdx.x] = (float)hist[threadIdx.x] / (float)(ns * nwin);
  if (threadIdx.x == 0) {
    f[0] = asinhf((float)(wc.alpha * 1000.0)) * 0.125f;
    f[1] = asinhf((float)(wc.mu * 1000.0)) * 0.125f;
    f[2] = asinhf((float)(wc.sigma * 1000.0)) * 0.125f;
  }
}

// Proposals of the batch's windows (W <= 32: one block) into d.prop; the
// narrow search of each window starts from them (launch_search_hint).
__global__ void __launch_bounds__(lam::H) k_lambda_propose(Problem pb, DeviceBuffers d) {
  extern __shared__ float smraw[];
  lam::Smem& sm = *reinterpret_cast<lam::Smem*>(smraw);
  const float* m = d.model;
  const __nv_bfloat16* wbf = (const __nv_bfloat16*)d.model_bf16;
  const int ns = min(pb.W, lam::SB);
  lam::load_inputs(m, d.feat, nullptr, 0, ns, sm);
  lam::forward(m, wbf, sm);
  if (threadIdx.x < ns) {
    const int w = threadIdx.x;
    const float y = sm.o[w] * m[lam::OFF_YSCALE] + m[lam::OFF_YMEAN];
    d.prop[w] = y;
    if (d.prop_out) d.prop_out[d.win0 + w] = y;
  }
}

size_t lambda_smem() { return sizeof(lam::Smem); }

cudaError_t launch_lambda_features(const Problem& pb, const DeviceBuffers& d, cudaStream_t s) {
  k_lambda_features<<<pb.W, 256, 0, s>>>(pb, d);
  return cudaGetLastError();
}

cudaError_t launch_lambda_propose(const Problem& pb, const DeviceBuffers& d, cudaStream_t s) {
  const size_t shm = lambda_smem();
  cudaError_t e = cudaFuncSetAttribute(k_lambda_propose, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)shm);
  if (e != cudaSuccess) return e;
  k_lambda_propose<<<1, lam::H, shm, s>>>(pb, d);
  return cudaGetLastError();
}

// ---- training / inference launchers (device buffers)
cudaError_t lambda_shadow(const float* m, void* wbf, cudaStream_t s) {
  lam::k_mlp_shadow<<<64, 256, 0, s>>>(m, (__nv_bfloat16*)wbf);
  return cudaGetLastError();
}

cudaError_t lambda_forward(const float* m, const void* wbf, const float* feat, int n, float* y,
                           cudaStream_t s) {
  const size_t shm = lambda_smem();
  cudaError_t e = cudaFuncSetAttribute(lam::k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)shm);
  if (e != cudaSuccess) return e;
  lam::k_mlp_forward<<<(n + lam::SB - 1) / lam::SB, lam::H, shm, s>>>(
      m, (const __nv_bfloat16*)wbf, feat, n, y);
  return cudaGetLastError();
}

cudaError_t lambda_grad(const float* m, const void* wbf, const float* feat, const float* target,
                        int n, float* part, float* part_loss, float* grad, cudaStream_t s) {
  const size_t shm = lambda_smem();
  cudaError_t e = cudaFuncSetAttribute(lam::k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)shm);
  if (e != cudaSuccess) return e;
  const int nblk = (n + lam::SB - 1) / lam::SB;
  lam::k_mlp_grad<<<nblk, lam::H, shm, s>>>(m, (const __nv_bfloat16*)wbf, feat, target, nullptr,
                                            nullptr, 0, 0, n, 1.f / (float)n, part, part_loss);
  lam::k_mlp_gsum<<<(lam::NPARAM + 255) / 256, 256, 0, s>>>(part, nblk, grad);
  return cudaGetLastError();
}

cudaError_t lambda_attrs() {
  const int shm = (int)lambda_smem();
  cudaError_t e = cudaFuncSetAttribute(lam::k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, shm);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(lam::k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, shm);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_lambda_propose, cudaFuncAttributeMaxDynamicSharedMemorySize, shm);
  return e;
}

// One epoch of training (stream-capturable: launches only; lambda_attrs()
// must have run).
cudaError_t lambda_train_epoch(const LambdaTrain& t, cudaStream_t s) {
  const size_t shm = lambda_smem();
  const int nblk = t.batch / lam::SB;
  lam::AdamCfg c{t.lr, t.lr_final, t.wd, t.b1, t.b2, t.eps, t.steps, t.total_steps};
  for (int st = 0; st < t.steps; ++st) {
    lam::k_mlp_grad<<<nblk, lam::H, shm, s>>>(
        t.m, (const __nv_bfloat16*)t.wbf, t.feat, t.target, t.perm, t.epoch, t.n, st * t.batch,
        t.n, 1.f / (float)t.batch, t.part, t.loss_acc + (size_t)st * nblk);
    lam::k_mlp_adam<<<(lam::NPARAM + 255) / 256, 256, 0, s>>>(t.m, (__nv_bfloat16*)t.wbf, t.mom1,
                                                            t.mom2, t.part, nblk, t.epoch, st, c);
  }
  lam::k_mlp_epoch_end<<<1, 32, 0, s>>>(t.loss_acc, t.steps, nblk, t.steps * t.batch, t.epoch,
                                        t.epoch_loss);
  return cudaGetLastError();
}

}  // namespace pgsvt
