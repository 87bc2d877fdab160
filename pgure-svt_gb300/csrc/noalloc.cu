// noalloc.cu — pgsvt_svd_window_noalloc: singular values of one window's
// Casorati matrices without any device allocation.
//
// Some callers cannot allocate device memory during their work: real-time
// acquisition loops that fixed their memory up front, code running under an
// external allocator that owns every byte of the device, or processes that
// must not call cudaMalloc/cudaFree because those calls synchronise the
// device.  For them this entry point takes caller-owned device inputs and
// outputs and keeps every intermediate in one file-scope device array of a
// fixed size (kScratchBytes, about 1 MB), which every GPU that loads the
// library holds until the process exits.  Windows larger than the limit are
// rejected.  All calls share the array, which keeps the last call's contents;
// calls whose GPU work overlaps (other host threads, other streams) race on
// it and must be serialised by the caller.
#include <cuda.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "pgsvt.h"
#include "pgsvt_internal.h"

namespace pgsvt {

namespace {

constexpr int kMaxSide = PGSVT_NOALLOC_MAX_SIDE;
constexpr int kMaxNwin = PGSVT_NOALLOC_MAX_NWIN;
constexpr int kMaxBs = 4;
constexpr int kMaxP = (kMaxSide - 2 + 1) * (kMaxSide - 2 + 1);  // bs >= 2
constexpr int kMaxNC = 16;

// carve-up of the scratch array (offsets in bytes, 256-byte aligned)
constexpr size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr size_t kOffPos = 0;
constexpr size_t kOffPlist = kOffPos + align256(sizeof(uint32_t) * kMaxNwin * kMaxP);
constexpr size_t kOffSv = kOffPlist + align256(sizeof(int32_t) * kMaxP);
constexpr size_t kOffHv = kOffSv + align256(sizeof(float) * kMaxNC * kMaxP);
constexpr size_t kOffNlive = kOffHv + align256(sizeof(float) * kMaxNC * kMaxP);
constexpr size_t kOffWc = kOffNlive + align256(sizeof(int32_t) * kMaxP);
constexpr size_t kOffCnt = kOffWc + align256(sizeof(WinConst));
constexpr size_t kOffErr = kOffCnt + align256(sizeof(unsigned long long) * 4);
constexpr size_t kScratchBytes = kOffErr + align256(sizeof(int));

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// pack the caller's trajectory table; flag positions outside the frame
__global__ void k_pack_positions(const int32_t* rows, const int32_t* cols, int n, int lim,
                                 uint32_t* pos, int* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int r = rows[i], c = cols[i];
  if (r < 0 || c < 0 || r > lim || c > lim) {
    atomicOr(err, 1);
    pos[i] = 0u;
    return;
  }
  pos[i] = (uint32_t)r | ((uint32_t)c << 16);
}

// S[p][i] (reference patch order) from the kernel's column-major sv[i][p]
__global__ void k_export_sv(const float* sv, int NP, int NC, int nwin, float* S) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= NP) return;
  for (int i = 0; i < nwin; ++i) S[(size_t)p * nwin + i] = sv[(size_t)i * NP + p];
}

std::mutex g_mu;
void* g_addr[64];                // scratch address per device, resolved on first use ...
unsigned long long g_ctx[64];    // ... in the context with this identifier

// Identifier of the calling thread's current CUDA context (0: none yet).  A
// device reset destroys the context that held the scratch and a new one gets
// a new identifier, so the address is resolved again after a reset.  The
// driver entry points are looked up through the runtime (no libcuda link).
unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = (GetCurrent)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = (GetId)f;
  });
  if (!get_current || !get_id) return 0;
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
  if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

int fail(int code, const std::string& m) {
  set_last_error(m);  // read back with pgsvt_last_error()
  return code;
}

}  // namespace
}  // namespace pgsvt

using namespace pgsvt;

extern "C" int pgsvt_svd_window_noalloc(const float* u_dev, uint32_t nrows, uint32_t nwin,
                                        uint32_t block_size, uint32_t block_overlap,
                                        const int32_t* rows_dev, const int32_t* cols_dev,
                                        float* S_dev, uint32_t* npatch, void* stream) {
  if (!u_dev || !rows_dev || !cols_dev || !npatch)
    return fail(PGSVT_ERR_INVALID_ARG, "null pointer");
  if (nrows < block_size || block_size < 2 || block_size > (uint32_t)kMaxBs)
    return fail(PGSVT_ERR_INVALID_ARG, "block_size must be in [2, 4] and at most the frame side");
  if (nrows > (uint32_t)kMaxSide || nwin > (uint32_t)kMaxNwin)
    return fail(PGSVT_ERR_INVALID_ARG,
                "window larger than the no-allocation limit (side <= " +
                    std::to_string(kMaxSide) + ", frames <= " + std::to_string(kMaxNwin) + ")");
  if (nwin % 2 == 0 || block_size * block_size <= nwin)
    return fail(PGSVT_ERR_INVALID_ARG, "nwin must be odd and below block_size^2");
  if (block_overlap < 1 || block_overlap > block_size)
    return fail(PGSVT_ERR_INVALID_ARG, "block_overlap out of range");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return fail(PGSVT_ERR_CUDA, "no usable CUDA device");
  // one-time set-up per device (the device is current): the host-side name
  // g_scratch is not a device address, ask the runtime for it; again when the
  // device's context has changed since (after a cudaDeviceReset)
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    const unsigned long long ctx = current_context_id();
    if (!g_addr[dev] || ctx == 0 || ctx != g_ctx[dev]) {
      const cudaError_t e = cudaGetSymbolAddress(&g_addr[dev], g_scratch);
      if (e != cudaSuccess) {
        g_addr[dev] = nullptr;
        return fail(PGSVT_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      }
      g_ctx[dev] = current_context_id();  // the set-up made the context current
    }
    base = g_addr[dev];
  }
  unsigned char* sb = (unsigned char*)base;
  cudaStream_t s = (cudaStream_t)stream;

  // geometry and the kept patches in the reference's sorted order
  Geometry g;
  g.S = (int)nrows;
  g.bs = (int)block_size;
  g.M = g.bs * g.bs;
  g.nwin = (int)nwin;
  g.fw = g.nwin / 2;
  g.Ntc = g.nwin;
  g.P = (g.S - g.bs + 1) * (g.S - g.bs + 1);
  g.NC = svd_columns(g.nwin);
  g.mw = 0;
  g.nimg = g.nwin;
  const std::vector<int32_t> plist = kept_patches(g.S, g.bs, (int)block_overlap);
  g.NP = (int)plist.size();
  *npatch = (uint32_t)g.NP;
  if (!S_dev) return PGSVT_OK;  // size query

  Problem pb{};
  pb.g = g;
  pb.W = 1;
  pb.K = 1;
  pb.optimize = 0;     // singular values only: an infinite flat threshold keeps no
  pb.expw = 0;         // triplet (not even an infinite singular value), so no
  pb.lambda_user = INFINITY;  // U/V factors are written (d.U0, d.V0 stay null)
  pb.compat = PGSVT_COMPAT_ALL;
  DeviceBuffers d{};
  d.u = const_cast<float*>(u_dev);
  d.pos = (uint32_t*)(sb + kOffPos);
  d.plist = (const int32_t*)(sb + kOffPlist);
  d.sv = (float*)(sb + kOffSv);
  d.hv = (float*)(sb + kOffHv);
  d.nlive0 = (int32_t*)(sb + kOffNlive);
  d.wc = (WinConst*)(sb + kOffWc);
  d.counters = (unsigned long long*)(sb + kOffCnt);
  int* err = (int*)(sb + kOffErr);
  d.ncopies = 1;

  // state left by the previous call: clear what must start at zero
  cudaError_t e = cudaMemsetAsync(sb + kOffWc, 0, kOffErr + sizeof(int) - kOffWc, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(sb + kOffPlist, plist.data(), sizeof(int32_t) * g.NP,
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    const int n = g.nwin * g.P;
    k_pack_positions<<<(n + 255) / 256, 256, 0, s>>>(rows_dev, cols_dev, n, g.S - g.bs, d.pos, err);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = launch_svd(pb, d, s);
  if (e == cudaSuccess) {
    k_export_sv<<<(g.NP + 255) / 256, 256, 0, s>>>(d.sv, g.NP, g.NC, g.nwin, S_dev);
    e = cudaGetLastError();
  }
  int herr = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // plist (host) must outlive the copy
  if (e != cudaSuccess) return fail(PGSVT_ERR_CUDA, cudaGetErrorString(e));
  if (herr) return fail(PGSVT_ERR_INVALID_ARG, "trajectory position outside the frame");
  set_last_error("");
  return PGSVT_OK;
}
