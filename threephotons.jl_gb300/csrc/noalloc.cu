// Bayes energy of a model correlation already in device memory, computed without
// allocating any device memory.
//
// Who needs this: callers that hold no right to allocate device memory at the moment
// they score a proposal.  A Julia host whose CUDA.jl memory pool owns the device
// memory is one: a foreign cudaMalloc may find the pool has taken nearly all of HBM,
// and cudaMalloc/cudaFree synchronise the device in the middle of the annealing loop.
// A host runtime with a fixed device-memory budget granted up front, or a real-time
// loop that must not stall on those implicit synchronisations, is another.  Such a
// caller passes its own device buffers for inputs and output; the per-slab scratch
// lives in the file-scope array below, which every GPU that loads this library holds
// until the process exits.
//
// The computation is the per-slab Bayes term and the deterministic compensated sum
// of the tensor-core path (the slab-energy epilogue and k_finalize_slabs), fed from a
// stored c3 instead of the accumulator in TMEM:
//   E = sum_ki tf(k1,k2,k3) * (Qs * log(sum_g p) - sum_g q^ log p),  p = max(c3, 1e-30),
//   Qs = sum_g q^  (q^ = the L1-normalised histogram slab).
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "../../include/tp3.h"
#include "internal.h"

namespace {

// Largest number of (k1 >= k2 >= k3) slabs one call may score: K <= 72.
constexpr int kNoAllocMaxSlabs = 65536;
constexpr int kMaxDevices = 64;

// Shared by every call on a device; each call overwrites every entry it later reads.
static __device__ __align__(256) double g_slab_energy[kNoAllocMaxSlabs];

// Device address of g_slab_energy per device ordinal, with the unique id of the
// context it was resolved in: a device reset (or a switch to another context on the
// same device) loads the module anew, possibly at another address, so the address is
// looked up again whenever the current context's id differs.
struct ScratchSlot {
  unsigned long long ctx_id;
  double* ptr;
};
std::mutex g_mu;
ScratchSlot g_scratch[kMaxDevices] = {};

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_current = nullptr;
CtxGetIdFn g_ctx_id = nullptr;
bool g_ctx_fns_tried = false;

// Unique id of the calling thread's current context (0 when there is none or the
// driver does not provide the query).  Called with g_mu held.
unsigned long long current_ctx_id() {
  if (!g_ctx_fns_tried) {
    g_ctx_fns_tried = true;
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
        q1 == cudaDriverEntryPointSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
        q2 == cudaDriverEntryPointSuccess) {
      g_ctx_current = (CtxGetCurrentFn)f1;
      g_ctx_id = (CtxGetIdFn)f2;
    }
  }
  if (!g_ctx_current || !g_ctx_id) return 0;
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (g_ctx_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
  if (g_ctx_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
  s = a + b;
  const double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// grid: klength; block 256.  One slab per block.
__global__ void __launch_bounds__(256) k_bayes_slab_noalloc(const float* __restrict__ c3,
                                                            const float* __restrict__ q, int klength, int G,
                                                            double* __restrict__ slab) {
  __shared__ double s_sp[256], s_sq[256], s_qs[256];
  const int ki = blockIdx.x;
  const float* cr = c3 + (size_t)ki * G;
  const float* qr = q + (size_t)ki * G;
  double sp = 0.0, sq = 0.0, qs = 0.0;
  for (int g = threadIdx.x; g < G; g += blockDim.x) {
    const float p = fmaxf(cr[g], 1e-30f);
    const float qv = qr[g];
    sp += (double)p;
    sq += (double)qv * (double)logf(p);
    qs += (double)qv;
  }
  s_sp[threadIdx.x] = sp;
  s_sq[threadIdx.x] = sq;
  s_qs[threadIdx.x] = qs;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      s_sp[threadIdx.x] += s_sp[threadIdx.x + h];
      s_sq[threadIdx.x] += s_sq[threadIdx.x + h];
      s_qs[threadIdx.x] += s_qs[threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    // slab ki -> (k1, k2, k3), k1 >= k2 >= k3, k1 outermost (src/correlations.jl:72-81)
    int k1 = 0, r = ki;
    while (r >= (k1 + 1) * (k1 + 2) / 2) { r -= (k1 + 1) * (k1 + 2) / 2; ++k1; }
    int k2 = 0;
    while (r >= k2 + 1) { r -= k2 + 1; ++k2; }
    const int k3 = r;
    const double tf = (k1 == k2 && k2 == k3) ? 1.0 : ((k1 == k2 || k1 == k3 || k2 == k3) ? 3.0 : 6.0);
    slab[ki] = tf * (s_qs[0] * log(s_sp[0]) - s_sq[0]);
  }
}

// grid: 1; block 256.  Deterministic compensated sum of the slab energies.
__global__ void __launch_bounds__(256) k_sum_slabs_noalloc(const double* __restrict__ slab, int klength,
                                                           double* __restrict__ E) {
  __shared__ double ss[256], sc[256];
  double s = 0.0, c = 0.0;
  for (int ki = threadIdx.x; ki < klength; ki += blockDim.x) {
    double t, err;
    two_sum(s, slab[ki], t, err);
    s = t;
    c += err;
  }
  ss[threadIdx.x] = s;
  sc[threadIdx.x] = c;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      double t, err;
      two_sum(ss[threadIdx.x], ss[threadIdx.x + h], t, err);
      ss[threadIdx.x] = t;
      sc[threadIdx.x] += sc[threadIdx.x + h] + err;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) E[0] = ss[0] + sc[0];
}

int noalloc_fail(int code, const std::string& msg) {
  tp3::set_thread_error(msg);  // reported by tp3_last_error(NULL)
  return code;
}

}  // namespace

extern "C" int tp3_bayes_energy_noalloc(const float* d_c3, const float* d_qhat, int K, int N, double* d_E,
                                        void* stream) {
  if (!d_c3 || !d_qhat || !d_E) return noalloc_fail(TP3_ERR_ARG, "NULL device pointer");
  if (K < 1 || N < 1) return noalloc_fail(TP3_ERR_ARG, "K and N must be >= 1");
  const long long klength = (long long)K * (K + 1) * (K + 2) / 6;
  if (klength > kNoAllocMaxSlabs)
    return noalloc_fail(TP3_ERR_ARG, "K too large: more than 65536 shell triples (K <= 72) for the static scratch");
  const long long G = 2LL * N * N;
  if (G > (1LL << 30)) return noalloc_fail(TP3_ERR_ARG, "N too large");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail(TP3_ERR_NO_DEVICE, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(TP3_ERR_NO_DEVICE, "device ordinal out of range");
  // an error left by the caller's earlier work would otherwise surface after this
  // call's launches and be reported as theirs: report it as what it is, uncleared
  e = cudaPeekAtLastError();
  if (e != cudaSuccess)
    return noalloc_fail(TP3_ERR_CUDA, std::string("an earlier CUDA error is pending (left uncleared): ") +
                                          cudaGetErrorString(e));
  double* scratch = nullptr;
  {
    // set-up on the first call in each context: resolve the device address of the
    // static array (cudaGetSymbolAddress loads the module into the current context)
    std::lock_guard<std::mutex> lock(g_mu);
    ScratchSlot& slot = g_scratch[dev];
    const unsigned long long id = current_ctx_id();
    if (!slot.ptr || id == 0 || slot.ctx_id != id) {
      double* p = nullptr;
      e = cudaGetSymbolAddress((void**)&p, g_slab_energy);
      if (e != cudaSuccess) {
        slot.ptr = nullptr;
        return noalloc_fail(TP3_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      }
      slot.ptr = p;
      slot.ctx_id = id != 0 ? id : current_ctx_id();  // the context exists now
    }
    scratch = slot.ptr;
  }
  cudaStream_t s = (cudaStream_t)stream;
  k_bayes_slab_noalloc<<<(unsigned)klength, 256, 0, s>>>(d_c3, d_qhat, (int)klength, (int)G, scratch);
  e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail(TP3_ERR_CUDA, std::string("slab launch: ") + cudaGetErrorString(e));
  k_sum_slabs_noalloc<<<1, 256, 0, s>>>(scratch, (int)klength, d_E);
  e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail(TP3_ERR_CUDA, std::string("sum launch: ") + cudaGetErrorString(e));
  return TP3_OK;
}
