// Learned proposal network (3 hidden layers, ReLU; BF16 weights and activations,
// FP32 accumulation) trained on the device by its own forward and backward kernels.
//
// Every matrix product is one tcgen05 kernel, k_gemm_tn: C[M][N] = A[M][K] B[N][K]^T
// with both operands K-major BF16 staged by TMA (64-byte swizzle, 4-stage mbarrier
// ring), one thread issuing tcgen05.mma (M = 128, N = BN, K = 16) into a TMEM
// accumulator, and four epilogue warps that read it with tcgen05.ld and apply
// bias, ReLU, the ReLU gate of the backward pass and up to three stores: BF16
// row-major, BF16 transposed (coalesced: TMEM lane = row) and FP32.
//
// Forward (rows R):   H1 = relu(X W1^T + b1), H2, H3 likewise, O = H3 W4^T + b4.
// Backward of the weighted Gaussian negative log-likelihood of logged steps v:
//   dO = d(sum_r w_r NLL_r)/dO (k_head_loss), dW4 = dO^T H3, dZ3 = (dO W4) . [H3 > 0],
//   dW3 = dZ3^T H2, dZ2 = (dZ3 W3) . [H2 > 0], dW2 = dZ2^T H1, dZ1 = (dZ2 W2) . [H1 > 0],
//   dW1 = dZ1^T X, db = column sums.  Transposed activations (H^T, dZ^T) written by
// the epilogues make every product a K-major x K-major tcgen05 product.
// Adam on FP32 master weights; BF16 copies W and W^T are refreshed after each step.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "ctx_internal.h"
#include "mlp.h"
#include "tc_prims.cuh"

namespace tp3 {
namespace {

constexpr int kGStages = 4;
constexpr int kGBM = 128;
constexpr int kGBK = 32;  // bf16 per 64-byte swizzled row
constexpr int kGThreads = 192;  // TMA warp, MMA warp, 4 epilogue warps
constexpr int kGABytes = kGBM * kGBK * 2;

struct GemmArgs {
  int M, N, K;
  const float* bias;            // [N] or null
  int relu;
  const __nv_bfloat16* gate;    // multiply by (gate[m * ldg + n] > 0) when non-null
  int ldg;
  __nv_bfloat16* out_bf;        // [M][ldo]
  int ldo;
  __nv_bfloat16* outT_bf;       // [N][ldt]
  int ldt;
  float* out_f32;               // [M][ldf]
  int ldf;
  int ksplit;                   // > 1: grid.z splits K; out_f32 accumulated with atomics (pre-zeroed)
  int* err;
};

struct GemmSmemHeader {
  uint64_t full[kGStages];
  uint64_t empty[kGStages];
  uint64_t tmem_full;
  uint32_t tmem_base;
  int abort_flag;
};

template <int BN>
__host__ __device__ constexpr int gemm_stage_bytes() { return kGABytes + BN * kGBK * 2; }
template <int BN>
constexpr size_t gemm_smem_bytes() { return 1024 + (size_t)kGStages * gemm_stage_bytes<BN>() + sizeof(GemmSmemHeader); }

// grid: (ceil(M / 128), ceil(N / BN)); block kGThreads.
template <int BN>
__global__ void __launch_bounds__(kGThreads, 1) k_gemm_tn(const __grid_constant__ CUtensorMap tmA,
                                                          const __grid_constant__ CUtensorMap tmB, GemmArgs g) {
  constexpr int kStage = gemm_stage_bytes<BN>();
  constexpr uint32_t kCols = BN < 32 ? 32u : (uint32_t)BN;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  GemmSmemHeader* hd = (GemmSmemHeader*)(base + kGStages * kStage);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * kGBM, n0 = blockIdx.y * BN;
  const int nk_all = (g.K + kGBK - 1) / kGBK;
  // split K: this CTA reduces k-blocks [kb0, kb0 + nk)
  const int ks = g.ksplit > 1 ? g.ksplit : 1;
  const int kb0 = (int)(((long long)nk_all * blockIdx.z) / ks);
  const int nk = (int)(((long long)nk_all * (blockIdx.z + 1)) / ks) - kb0;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kGStages; ++s) {
      mbar_init(&hd->full[s], 1);
      mbar_init(&hd->empty[s], 1);
    }
    mbar_init(&hd->tmem_full, 1);
    hd->abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&hd->tmem_base)),
                 "r"(kCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = hd->tmem_base;
  volatile int* abort_flag = &hd->abort_flag;

  if (warp == 0) {
    if (lane == 0) {
      int last[kGStages];
#pragma unroll
      for (int s = 0; s < kGStages; ++s) last[s] = -1;
      for (int kc = 0; kc < nk; ++kc) {
        const int s = kc % kGStages;
        const uint32_t ph = (uint32_t)((kc / kGStages) & 1);
        if (!mbar_wait(&hd->empty[s], ph ^ 1u, abort_flag, g.err)) break;
        last[s] = kc;
        uint8_t* st = base + s * kStage;
        mbar_expect_tx(&hd->full[s], kStage);
        tma_load_2d(st, &tmA, &hd->full[s], (kb0 + kc) * kGBK, m0);
        tma_load_2d(st + kGABytes, &tmB, &hd->full[s], (kb0 + kc) * kGBK, n0);
      }
      if (*abort_flag) {
        for (int s = 0; s < kGStages; ++s) {
          if (last[s] < 0) continue;
          const long long t0 = clock64();
          while (!mbar_try_wait(&hd->full[s], (uint32_t)((last[s] / kGStages) & 1)) && clock64() - t0 < kTimeoutCycles) {
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                             ((uint32_t)(kGBM >> 4) << 24);
      bool ok = true;
      for (int kc = 0; kc < nk; ++kc) {
        const int s = kc % kGStages;
        const uint32_t ph = (uint32_t)((kc / kGStages) & 1);
        if (!mbar_wait(&hd->full[s], ph, abort_flag, g.err)) { ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t st = smem_u32(base + s * kStage);
        const uint64_t ad = smem_desc_sw64(st), bd = smem_desc_sw64(st + kGABytes);
#pragma unroll
        for (int ks = 0; ks < 2; ++ks)
          mma_issue<false>(tmem, ad + (uint64_t)(ks * 2), bd + (uint64_t)(ks * 2), idesc, (kc > 0 || ks > 0) ? 1u : 0u);
        mma_commit(&hd->empty[s]);
      }
      if (ok) mma_commit(&hd->tmem_full);
    }
  } else {
    const int q = warp & 3;  // TMEM lane quarter this warp may read
    const int r = q * 32 + lane;
    const int m = m0 + r;
    if (nk > 0 && mbar_wait(&hd->tmem_full, 0u, abort_flag, g.err)) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int c = 0; c < (BN + 31) / 32; ++c) {
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(c * 32), v);
        const int nb = n0 + c * 32;
        // a whole 32-column run inside the tile and the matrix: 16-byte vector loads/stores
        const bool full = c * 32 + 32 <= BN && nb + 32 <= g.N && (!g.out_bf || g.ldo % 8 == 0) &&
                          (!g.gate || g.ldg % 8 == 0);
        if (m < g.M && full) {
          float x[32];
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            x[j] = v[j];
            if (g.bias) x[j] += g.bias[nb + j];
            if (g.relu) x[j] = fmaxf(x[j], 0.f);
          }
          if (g.gate) {
            const uint4* gp = reinterpret_cast<const uint4*>(g.gate + (size_t)m * g.ldg + nb);
#pragma unroll
            for (int q4 = 0; q4 < 4; ++q4) {
              const uint4 u = gp[q4];
              const uint32_t w4[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
              for (int t = 0; t < 4; ++t) {
                const __nv_bfloat162 h = *reinterpret_cast<const __nv_bfloat162*>(&w4[t]);
                if (!(__low2float(h) > 0.f)) x[q4 * 8 + 2 * t] = 0.f;
                if (!(__high2float(h) > 0.f)) x[q4 * 8 + 2 * t + 1] = 0.f;
              }
            }
          }
          if (g.out_f32) {
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              if (ks > 1) atomicAdd(&g.out_f32[(size_t)m * g.ldf + nb + j], x[j]);
              else g.out_f32[(size_t)m * g.ldf + nb + j] = x[j];
            }
          }
          if (g.out_bf) {
            uint4* op = reinterpret_cast<uint4*>(g.out_bf + (size_t)m * g.ldo + nb);
#pragma unroll
            for (int q4 = 0; q4 < 4; ++q4) {
              uint32_t w4[4];
#pragma unroll
              for (int t = 0; t < 4; ++t) {
                const __nv_bfloat162 h = __floats2bfloat162_rn(x[q4 * 8 + 2 * t], x[q4 * 8 + 2 * t + 1]);
                w4[t] = *reinterpret_cast<const uint32_t*>(&h);
              }
              op[q4] = make_uint4(w4[0], w4[1], w4[2], w4[3]);
            }
          }
          if (g.outT_bf) {
#pragma unroll
            for (int j = 0; j < 32; ++j) g.outT_bf[(size_t)(nb + j) * g.ldt + m] = __float2bfloat16_rn(x[j]);
          }
        } else if (m < g.M) {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int n = nb + j;
            if (c * 32 + j >= BN || n >= g.N) continue;
            float x = v[j];
            if (g.bias) x += g.bias[n];
            if (g.relu) x = fmaxf(x, 0.f);
            if (g.gate && !(__bfloat162float(g.gate[(size_t)m * g.ldg + n]) > 0.f)) x = 0.f;
            if (g.out_f32) {
              if (ks > 1) atomicAdd(&g.out_f32[(size_t)m * g.ldf + n], x);
              else g.out_f32[(size_t)m * g.ldf + n] = x;
            }
            const __nv_bfloat16 xb = __float2bfloat16_rn(x);
            if (g.out_bf) g.out_bf[(size_t)m * g.ldo + n] = xb;
            if (g.outT_bf) g.outT_bf[(size_t)n * g.ldt + m] = xb;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols) : "memory");
  }
}

// X [R][ld] -> Xt [C][ldt]; grid (ceil(C/32), ceil(R/32)), block (32, 8).
__global__ void k_transpose_bf16(const __nv_bfloat16* __restrict__ X, int R, int C, int ld, __nv_bfloat16* __restrict__ Xt,
                                 int ldt) {
  __shared__ __nv_bfloat16 t[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += 8) {
    const int r = r0 + i, c = c0 + threadIdx.x;
    t[i][threadIdx.x] = (r < R && c < C) ? X[(size_t)r * ld + c] : __float2bfloat16_rn(0.f);
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += 8) {
    const int c = c0 + i, r = r0 + threadIdx.x;
    if (c < C && r < R) Xt[(size_t)c * ldt + r] = t[threadIdx.x][i];
  }
}

// Regression of the logged energy changes on the steps: for candidate j (rows
// jK..jK+K-1, one per shell) r_j = t_j - sum_k u_k . V_k with (t_j, lambda_j) = tw[j],
// V = v / sigma the logged step; resid[j] = lambda_j r_j, part[block] = sum of
// lambda_j r_j^2 / 2.  grid ceil(nc / 128), block 128.
__global__ void k_reg_residual(const float* __restrict__ O, const float* __restrict__ V,
                               const float2* __restrict__ tw, int K, int nc, float* __restrict__ resid,
                               double* __restrict__ part) {
  __shared__ double red[128];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  double l = 0.0;
  if (j < nc) {
    double p = 0.0;
    for (int k = 0; k < K; ++k) {
      const size_t r = (size_t)j * K + k;
      for (int d = 0; d < 3; ++d) p += (double)O[r * kMlpOutPad + d] * (double)V[r * 3 + d];
    }
    const float2 t = tw[j];
    const double res = (double)t.x - p;
    resid[j] = (float)((double)t.y * res);
    l = 0.5 * (double)t.y * res * res;
  }
  red[threadIdx.x] = l;
  __syncthreads();
  for (int h = 64; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// Gradient of the loss wrt the raw outputs: the regression term on u (resid
// nullable: none) and the weighted zero-mean Gaussian NLL of the logged steps V on
// the log-scales s, sum_d w [s_d + V_d^2 exp(-2 s_d) / 2 + log(2 pi) / 2].
// grid ceil(R/128), block 128.  dO [R][16] bf16 and dOt [16][ldt] bf16 (columns /
// rows 6..15 zero); part[block] = sum of w NLL over the block.
__global__ void k_head_loss(const float* __restrict__ O, int R, const float* __restrict__ vlog,
                            const float* __restrict__ w, const float* __restrict__ resid, int K, int nc,
                            __nv_bfloat16* __restrict__ dO, __nv_bfloat16* __restrict__ dOt, int ldt,
                            double* __restrict__ part) {
  __shared__ double red[128];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  double nll = 0.0;
  if (r < R) {
    const float* o = O + (size_t)r * kMlpOutPad;
    const double wr = w[r];
    const double rj = (resid && r / K < nc) ? (double)resid[r / K] : 0.0;
    float g[kMlpOutPad];
    for (int j = 0; j < kMlpOutPad; ++j) g[j] = 0.f;
    for (int d = 0; d < 3; ++d) {
      const double ts = tanh((double)o[3 + d]);
      const double s = kSMid + kSHalf * ts;
      const double e = (double)vlog[(size_t)r * 3 + d];
      const double is2 = exp(-2.0 * s);
      nll += s + 0.5 * e * e * is2 + 0.9189385332046727;  // 0.5 log(2 pi)
      g[d] = (float)(-rj * e);
      g[3 + d] = (float)(wr * (1.0 - e * e * is2) * kSHalf * (1.0 - ts * ts));
    }
    nll *= wr;
    for (int j = 0; j < kMlpOutPad; ++j) {
      const __nv_bfloat16 b = __float2bfloat16_rn(g[j]);
      dO[(size_t)r * kMlpOutPad + j] = b;
      dOt[(size_t)j * ldt + r] = b;
    }
  }
  red[threadIdx.x] = nll;
  __syncthreads();
  for (int h = 64; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// db[n] = sum_r Zt[n][r] (FP32 sum of BF16 values); grid N, block 256.
__global__ void k_rowsum_bf16(const __nv_bfloat16* __restrict__ Zt, int ldt, int R, float* __restrict__ db) {
  __shared__ float red[256];
  const __nv_bfloat16* z = Zt + (size_t)blockIdx.x * ldt;
  float s = 0.f;
  for (int r = threadIdx.x; r < R; r += blockDim.x) s += __bfloat162float(z[r]);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) db[blockIdx.x] = red[0];
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       long long n, float lr, float b1, float b2, float eps, float c1, float c2) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// master W [out][in] (FP32) -> W_bf [out][ldw] and, when Wt, W^T [in][ldt] (BF16).
__global__ void k_pack_weights(const float* __restrict__ W, int out, int in, __nv_bfloat16* __restrict__ Wb, int ldw,
                               __nv_bfloat16* __restrict__ Wt, int ldt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= out * in) return;
  const int o = i / in, k = i - o * in;
  const __nv_bfloat16 b = __float2bfloat16_rn(W[i]);
  Wb[(size_t)o * ldw + k] = b;
  if (Wt) Wt[(size_t)k * ldt + o] = b;
}

// raw outputs -> (u, s) rows of 6; grid ceil(R/128), block 128
__global__ void k_head_map(const float* __restrict__ O, int R, float* __restrict__ out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  double u[3], s[3];
  mlp_head(O + (size_t)r * kMlpOutPad, u, s);
  for (int d = 0; d < 3; ++d) {
    out[(size_t)r * 6 + d] = (float)u[d];
    out[(size_t)r * 6 + 3 + d] = (float)s[d];
  }
}

uint64_t splitmix64(uint64_t& x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace
}  // namespace tp3

struct tp3_mlp {
  tp3_ctx* ctx = nullptr;
  int n_in = 0, n_in_pad = 0, H = 0, max_rows = 0;
  // FP32 master parameters [W1 (H x n_in), b1, W2 (H x H), b2, W3, b3, W4 (6 x H), b4]
  long long n_par = 0;
  long long off_W[4] = {}, off_b[4] = {};
  float* d_par = nullptr;
  float* d_grad = nullptr;
  float* d_m = nullptr;
  float* d_v = nullptr;
  long long adam_t = 0;
  // BF16 weight copies
  __nv_bfloat16 *W1 = nullptr, *W2 = nullptr, *W3 = nullptr, *W4 = nullptr;  // [out][in_pad]
  __nv_bfloat16 *W2t = nullptr, *W3t = nullptr, *W4t = nullptr;               // [in][out_pad]
  // activations
  __nv_bfloat16 *X = nullptr, *Xt = nullptr;     // [max_rows][n_in_pad], [n_in_pad][max_rows]
  __nv_bfloat16 *Hh[3] = {}, *Ht[3] = {};        // [max_rows][H], [H][max_rows]
  float* O = nullptr;                            // [max_rows][16]
  __nv_bfloat16 *dO = nullptr, *dOt = nullptr;   // [max_rows][16], [16][max_rows]
  __nv_bfloat16 *P = nullptr, *Q = nullptr, *Tt = nullptr;  // [max_rows][H] x2, [H][max_rows]
  double* d_part = nullptr;                      // loss partials [2][max_rows / 128] (NLL, regression)
  float* d_resid = nullptr;                      // weighted regression residual per candidate [max_rows]
  int* d_err = nullptr;
  // tensor maps: forward F1..F4, backward B1..B7
  CUtensorMap fA[4], fB[4], bA[7], bB[7];
};

namespace tp3 {
namespace {

cudaError_t enc(tp3_ctx* c, CUtensorMap* m, const void* ptr, uint64_t inner, uint64_t rows, uint64_t ld,
                uint32_t box_rows) {
  cuuint64_t dims[2] = {inner, rows};
  cuuint64_t strides[1] = {ld * 2};
  cuuint32_t box[2] = {(cuuint32_t)kGBK, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = c->encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, es,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

int pick_bn(int N) { return N <= 16 ? 16 : (N <= 128 ? 128 : 256); }

cudaError_t gemm(tp3_mlp* net, const CUtensorMap& A, const CUtensorMap& B, GemmArgs g) {
  const int bn = pick_bn(g.N);
  g.err = net->d_err;
  dim3 grid((g.M + kGBM - 1) / kGBM, (g.N + bn - 1) / bn);
  if (g.ksplit < 1) g.ksplit = 1;
  grid.z = g.ksplit;
  cudaStream_t s = net->ctx->stream;
  if (bn == 16) k_gemm_tn<16><<<grid, kGThreads, gemm_smem_bytes<16>(), s>>>(A, B, g);
  else if (bn == 128) k_gemm_tn<128><<<grid, kGThreads, gemm_smem_bytes<128>(), s>>>(A, B, g);
  else k_gemm_tn<256><<<grid, kGThreads, gemm_smem_bytes<256>(), s>>>(A, B, g);
  return cudaGetLastError();
}

GemmArgs args(int M, int N, int K) {
  GemmArgs g;
  std::memset(&g, 0, sizeof(g));
  g.M = M; g.N = N; g.K = K;
  return g;
}

void mlp_free(tp3_mlp* n) {
  void* ps[] = {n->d_par, n->d_grad, n->d_m, n->d_v, n->W1, n->W2, n->W3, n->W4, n->W2t, n->W3t, n->W4t, n->X, n->Xt,
                n->Hh[0], n->Hh[1], n->Hh[2], n->Ht[0], n->Ht[1], n->Ht[2], n->O, n->dO, n->dOt, n->P, n->Q, n->Tt,
                n->d_part, n->d_resid, n->d_err};
  for (void* p : ps) cudaFree(p);
}

cudaError_t pack_all(tp3_mlp* n) {
  cudaStream_t s = n->ctx->stream;
  const int H = n->H;
  struct L { long long off; int out, in; __nv_bfloat16* Wb; int ldw; __nv_bfloat16* Wt; int ldt; };
  const L ls[4] = {{n->off_W[0], H, n->n_in, n->W1, n->n_in_pad, nullptr, 0},
                   {n->off_W[1], H, H, n->W2, H, n->W2t, H},
                   {n->off_W[2], H, H, n->W3, H, n->W3t, H},
                   {n->off_W[3], kMlpOut, H, n->W4, H, n->W4t, kMlpOutPad}};
  for (const L& l : ls) {
    const int tot = l.out * l.in;
    k_pack_weights<<<(tot + 255) / 256, 256, 0, s>>>(n->d_par + l.off, l.out, l.in, l.Wb, l.ldw, l.Wt, l.ldt);
  }
  return cudaGetLastError();
}

// forward on rows [0, R) of the net's input buffer; the transposed activations the
// backward pass reads are written only when training (with_t)
cudaError_t forward(tp3_mlp* n, int R, bool with_t) {
  cudaError_t e;
  const int H = n->H;
  for (int l = 0; l < 3; ++l) {
    GemmArgs g = args(R, H, l == 0 ? n->n_in_pad : H);
    g.bias = n->d_par + n->off_b[l];
    g.relu = 1;
    g.out_bf = n->Hh[l]; g.ldo = H;
    if (with_t) { g.outT_bf = n->Ht[l]; g.ldt = n->max_rows; }
    if ((e = gemm(n, n->fA[l], n->fB[l], g)) != cudaSuccess) return e;
  }
  GemmArgs g = args(R, kMlpOut, H);
  g.bias = n->d_par + n->off_b[3];
  g.out_f32 = n->O; g.ldf = kMlpOutPad;
  return gemm(n, n->fA[3], n->fB[3], g);
}

// loss and gradient into d_grad for rows [0, R), R a multiple of 128; tw (nullable):
// per-candidate regression targets and weights of candidates of K rows each
cudaError_t backward(tp3_mlp* n, int R, const float* v, const float* w, const float* tw, int K) {
  cudaError_t e;
  cudaStream_t s = n->ctx->stream;
  const int H = n->H, MR = n->max_rows;
  dim3 tg((n->n_in_pad + 31) / 32, (R + 31) / 32), tb(32, 8);
  k_transpose_bf16<<<tg, tb, 0, s>>>(n->X, R, n->n_in_pad, n->n_in_pad, n->Xt, MR);
  const int nc = R / K;
  if (tw) {
    k_reg_residual<<<(nc + 127) / 128, 128, 0, s>>>(n->O, v, reinterpret_cast<const float2*>(tw), K, nc, n->d_resid,
                                                   n->d_part + MR / 128);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  k_head_loss<<<R / 128, 128, 0, s>>>(n->O, R, v, w, tw ? n->d_resid : nullptr, K, nc, n->dO, n->dOt, MR, n->d_part);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  float* gW[4];
  float* gb[4];
  for (int l = 0; l < 4; ++l) { gW[l] = n->d_grad + n->off_W[l]; gb[l] = n->d_grad + n->off_b[l]; }
  // weight gradients reduce over the R rows: split K so that about two CTAs per SM work
  if ((e = cudaMemsetAsync(n->d_grad, 0, n->n_par * sizeof(float), s)) != cudaSuccess) return e;
  auto split = [&](int M, int N) {
    const int tiles = ((M + kGBM - 1) / kGBM) * ((N + pick_bn(N) - 1) / pick_bn(N));
    const int nk = (R + kGBK - 1) / kGBK;
    int k = 304 / tiles;
    k = k < 1 ? 1 : k;
    k = k > nk / 4 ? (nk / 4 > 0 ? nk / 4 : 1) : k;
    return k;
  };
  // B1: dW4 = dO^T H3  [6 x H]
  GemmArgs g = args(kMlpOut, H, R);
  g.out_f32 = gW[3]; g.ldf = H; g.ksplit = split(kMlpOut, H);
  if ((e = gemm(n, n->bA[0], n->bB[0], g)) != cudaSuccess) return e;
  k_rowsum_bf16<<<kMlpOut, 256, 0, s>>>(n->dOt, MR, R, gb[3]);
  // B2: dZ3 = (dO W4) . [H3 > 0] -> P, Tt
  g = args(R, H, kMlpOutPad);
  g.gate = n->Hh[2]; g.ldg = H; g.out_bf = n->P; g.ldo = H; g.outT_bf = n->Tt; g.ldt = MR;
  if ((e = gemm(n, n->bA[1], n->bB[1], g)) != cudaSuccess) return e;
  // B3: dW3 = dZ3^T H2
  g = args(H, H, R);
  g.out_f32 = gW[2]; g.ldf = H; g.ksplit = split(H, H);
  if ((e = gemm(n, n->bA[2], n->bB[2], g)) != cudaSuccess) return e;
  k_rowsum_bf16<<<H, 256, 0, s>>>(n->Tt, MR, R, gb[2]);
  // B4: dZ2 = (dZ3 W3) . [H2 > 0] -> Q, Tt
  g = args(R, H, H);
  g.gate = n->Hh[1]; g.ldg = H; g.out_bf = n->Q; g.ldo = H; g.outT_bf = n->Tt; g.ldt = MR;
  if ((e = gemm(n, n->bA[3], n->bB[3], g)) != cudaSuccess) return e;
  // B5: dW2 = dZ2^T H1
  g = args(H, H, R);
  g.out_f32 = gW[1]; g.ldf = H; g.ksplit = split(H, H);
  if ((e = gemm(n, n->bA[4], n->bB[4], g)) != cudaSuccess) return e;
  k_rowsum_bf16<<<H, 256, 0, s>>>(n->Tt, MR, R, gb[1]);
  // B6: dZ1^T = ((dZ2 W2) . [H1 > 0])^T -> Tt
  g = args(R, H, H);
  g.gate = n->Hh[0]; g.ldg = H; g.outT_bf = n->Tt; g.ldt = MR;
  if ((e = gemm(n, n->bA[5], n->bB[5], g)) != cudaSuccess) return e;
  // B7: dW1 = dZ1^T X  [H x n_in]
  g = args(H, n->n_in, R);
  g.out_f32 = gW[0]; g.ldf = n->n_in; g.ksplit = split(H, n->n_in);
  if ((e = gemm(n, n->bA[6], n->bB[6], g)) != cudaSuccess) return e;
  k_rowsum_bf16<<<H, 256, 0, s>>>(n->Tt, MR, R, gb[0]);
  return cudaGetLastError();
}

}  // namespace

cudaError_t mlp_configure() {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(k_gemm_tn<16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)gemm_smem_bytes<16>())) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_gemm_tn<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)gemm_smem_bytes<128>())) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_gemm_tn<256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)gemm_smem_bytes<256>())) != cudaSuccess)
    return e;
  return cudaSuccess;
}

// Raw network outputs (before the head mapping) of rows [0, R) of the input buffer.
int mlp_forward_raw(tp3_mlp* n, int R, const float** out) {
  cudaError_t e = forward(n, R, false);
  if (e != cudaSuccess) return ctx_cuda_fail(n->ctx, e, "mlp forward");
  *out = n->O;
  return TP3_OK;
}

__nv_bfloat16* mlp_input(tp3_mlp* n) { return n->X; }
int mlp_max_rows(const tp3_mlp* n) { return n->max_rows; }
int mlp_n_in_of(const tp3_mlp* n) { return n->n_in; }

}  // namespace tp3

extern "C" {

int tp3_mlp_create(tp3_ctx* c, int n_in, int hidden, int max_rows, uint64_t seed, tp3_mlp** out) {
  if (int r = tp3::ctx_check(c)) return r;
  if (!out || n_in < 1 || hidden < 32 || hidden % 32 != 0 || hidden > 4096 || max_rows < 128 || max_rows % 128 != 0)
    return tp3::ctx_fail(c, TP3_ERR_ARG, "mlp needs n_in >= 1, hidden a multiple of 32 (<= 4096), max_rows a multiple of 128");
  if (!c->encode) return tp3::ctx_fail(c, TP3_ERR_UNSUPPORTED, "tensor-map encoder unavailable");
  *out = nullptr;
  static bool configured = false;
  if (!configured) {
    cudaError_t e = tp3::mlp_configure();
    if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "mlp configure");
    configured = true;
  }
  tp3_mlp* n = new tp3_mlp();
  n->ctx = c;
  n->n_in = n_in;
  n->n_in_pad = (n_in + 31) / 32 * 32;
  n->H = hidden;
  n->max_rows = max_rows;
  const int H = hidden, IP = n->n_in_pad, MR = max_rows;
  const int outs[4] = {H, H, H, tp3::kMlpOut}, ins[4] = {n_in, H, H, H};
  long long off = 0;
  for (int l = 0; l < 4; ++l) {
    n->off_W[l] = off; off += (long long)outs[l] * ins[l];
    n->off_b[l] = off; off += outs[l];
  }
  n->n_par = off;
  cudaError_t e = cudaSuccess;
  auto A = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) e = cudaMemsetAsync(*p, 0, bytes, c->stream);
  };
  const size_t bf = sizeof(__nv_bfloat16);
  A((void**)&n->d_par, off * 4); A((void**)&n->d_grad, off * 4); A((void**)&n->d_m, off * 4); A((void**)&n->d_v, off * 4);
  A((void**)&n->W1, (size_t)H * IP * bf); A((void**)&n->W2, (size_t)H * H * bf); A((void**)&n->W3, (size_t)H * H * bf);
  A((void**)&n->W4, (size_t)tp3::kMlpOutPad * H * bf);
  A((void**)&n->W2t, (size_t)H * H * bf); A((void**)&n->W3t, (size_t)H * H * bf);
  A((void**)&n->W4t, (size_t)H * tp3::kMlpOutPad * bf);
  A((void**)&n->X, (size_t)MR * IP * bf); A((void**)&n->Xt, (size_t)IP * MR * bf);
  for (int l = 0; l < 3; ++l) { A((void**)&n->Hh[l], (size_t)MR * H * bf); A((void**)&n->Ht[l], (size_t)H * MR * bf); }
  A((void**)&n->O, (size_t)MR * tp3::kMlpOutPad * 4);
  A((void**)&n->dO, (size_t)MR * tp3::kMlpOutPad * bf); A((void**)&n->dOt, (size_t)tp3::kMlpOutPad * MR * bf);
  A((void**)&n->P, (size_t)MR * H * bf); A((void**)&n->Q, (size_t)MR * H * bf); A((void**)&n->Tt, (size_t)H * MR * bf);
  A((void**)&n->d_part, (size_t)(2 * MR / 128) * sizeof(double)); A((void**)&n->d_err, sizeof(int));
  A((void**)&n->d_resid, (size_t)MR * sizeof(float));
  if (e != cudaSuccess) {
    tp3::mlp_free(n);
    delete n;
    cudaGetLastError();
    return tp3::ctx_fail(c, TP3_ERR_ALLOC, std::string("mlp allocation: ") + cudaGetErrorString(e));
  }
  // He-uniform initial weights (last layer scaled by 0.01 so the first outputs are
  // close to u = 0, s = kSMid); zero biases
  std::vector<float> par(off, 0.f);
  uint64_t st = seed ^ 0x6d6c7033ull;
  for (int l = 0; l < 4; ++l) {
    const double lim = std::sqrt(6.0 / ins[l]) * (l == 3 ? 0.01 : 1.0);
    for (long long i = 0; i < (long long)outs[l] * ins[l]; ++i) {
      const double u = (double)(tp3::splitmix64(st) >> 11) * (1.0 / 9007199254740992.0);
      par[n->off_W[l] + i] = (float)((2.0 * u - 1.0) * lim);
    }
  }
  // tensor maps
  const int hb = tp3::pick_bn(H), ib = tp3::pick_bn(n_in);
  bool ok = true;
  auto M = [&](CUtensorMap* m, const void* p, uint64_t inner, uint64_t rows, uint64_t ld, uint32_t box) {
    ok = ok && tp3::enc(c, m, p, inner, rows, ld, box) == cudaSuccess;
  };
  M(&n->fA[0], n->X, IP, MR, IP, 128);  M(&n->fB[0], n->W1, IP, H, IP, hb);
  M(&n->fA[1], n->Hh[0], H, MR, H, 128); M(&n->fB[1], n->W2, H, H, H, hb);
  M(&n->fA[2], n->Hh[1], H, MR, H, 128); M(&n->fB[2], n->W3, H, H, H, hb);
  M(&n->fA[3], n->Hh[2], H, MR, H, 128); M(&n->fB[3], n->W4, H, tp3::kMlpOutPad, H, 16);
  M(&n->bA[0], n->dOt, MR, tp3::kMlpOutPad, MR, 128); M(&n->bB[0], n->Ht[2], MR, H, MR, hb);
  M(&n->bA[1], n->dO, tp3::kMlpOutPad, MR, tp3::kMlpOutPad, 128); M(&n->bB[1], n->W4t, tp3::kMlpOutPad, H, tp3::kMlpOutPad, hb);
  M(&n->bA[2], n->Tt, MR, H, MR, 128); M(&n->bB[2], n->Ht[1], MR, H, MR, hb);
  M(&n->bA[3], n->P, H, MR, H, 128); M(&n->bB[3], n->W3t, H, H, H, hb);
  M(&n->bA[4], n->Tt, MR, H, MR, 128); M(&n->bB[4], n->Ht[0], MR, H, MR, hb);
  M(&n->bA[5], n->Q, H, MR, H, 128); M(&n->bB[5], n->W2t, H, H, H, hb);
  M(&n->bA[6], n->Tt, MR, H, MR, 128); M(&n->bB[6], n->Xt, MR, IP, MR, ib);
  if (!ok) {
    tp3::mlp_free(n);
    delete n;
    return tp3::ctx_fail(c, TP3_ERR_CUDA, "mlp tensor map encoding failed");
  }
  if ((e = cudaMemcpyAsync(n->d_par, par.data(), off * 4, cudaMemcpyHostToDevice, c->stream)) != cudaSuccess ||
      (e = tp3::pack_all(n)) != cudaSuccess || (e = cudaStreamSynchronize(c->stream)) != cudaSuccess) {
    tp3::mlp_free(n);
    delete n;
    return tp3::ctx_cuda_fail(c, e, "mlp init");
  }
  *out = n;
  return TP3_OK;
}

void tp3_mlp_destroy(tp3_mlp* n) {
  if (!n) return;
  cudaSetDevice(n->ctx->device);
  cudaStreamSynchronize(n->ctx->stream);
  tp3::mlp_free(n);
  delete n;
}

int tp3_mlp_num_params(const tp3_mlp* n, int64_t* count) {
  if (!n || !count) return TP3_ERR_ARG;
  *count = n->n_par;
  return TP3_OK;
}

int tp3_mlp_get_params(tp3_mlp* n, float* host, int64_t count) {
  if (!n || !host || count != n->n_par) return TP3_ERR_ARG;
  tp3_ctx* c = n->ctx;
  cudaError_t e = cudaMemcpyAsync(host, n->d_par, count * 4, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "mlp get params");
  return TP3_OK;
}

int tp3_mlp_set_params(tp3_mlp* n, const float* host, int64_t count) {
  if (!n || !host || count != n->n_par) return TP3_ERR_ARG;
  tp3_ctx* c = n->ctx;
  cudaError_t e = cudaMemcpyAsync(n->d_par, host, count * 4, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = tp3::pack_all(n);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "mlp set params");
  n->adam_t = 0;
  cudaMemsetAsync(n->d_m, 0, n->n_par * 4, c->stream);
  cudaMemsetAsync(n->d_v, 0, n->n_par * 4, c->stream);
  return TP3_OK;
}

int tp3_mlp_input_buffer(tp3_mlp* n, void** d_x, int* row_stride) {
  if (!n || !d_x || !row_stride) return TP3_ERR_ARG;
  *d_x = n->X;
  *row_stride = n->n_in_pad;
  return TP3_OK;
}

static int mlp_load_input(tp3_mlp* n, int rows, const void* d_x) {
  tp3_ctx* c = n->ctx;
  if (int r = tp3::ctx_check(c)) return r;
  if (rows < 1 || rows > n->max_rows || !d_x) return tp3::ctx_fail(c, TP3_ERR_ARG, "bad mlp rows or input");
  if (d_x != (const void*)n->X) {
    cudaError_t e = cudaMemcpyAsync(n->X, d_x, (size_t)rows * n->n_in_pad * sizeof(__nv_bfloat16),
                                    cudaMemcpyDeviceToDevice, c->stream);
    if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "mlp input copy");
  }
  return TP3_OK;
}

int tp3_mlp_forward_device(tp3_mlp* n, int rows, const void* d_x, void* d_out) {
  if (!n || !d_out) return TP3_ERR_ARG;
  if (int r = mlp_load_input(n, rows, d_x)) return r;
  tp3_ctx* c = n->ctx;
  cudaError_t e = tp3::forward(n, rows, false);
  if (e == cudaSuccess) {
    tp3::k_head_map<<<(rows + 127) / 128, 128, 0, c->stream>>>(n->O, rows, (float*)d_out);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "mlp forward");
  return TP3_OK;
}

static int mlp_loss_grad(tp3_mlp* n, int rows, const void* d_x, const float* d_v, const float* d_w,
                         const float* d_target, int shells, double* loss) {
  tp3_ctx* c = n->ctx;
  if (rows % 128 != 0) return tp3::ctx_fail(c, TP3_ERR_ARG, "training rows must be a multiple of 128");
  if (!d_v || !d_w) return tp3::ctx_fail(c, TP3_ERR_ARG, "NULL steps or weights");
  if (shells < 1 || shells > rows) return tp3::ctx_fail(c, TP3_ERR_ARG, "shells per candidate out of range");
  if (int r = mlp_load_input(n, rows, d_x)) return r;
  cudaError_t e = cudaMemsetAsync(n->d_err, 0, sizeof(int), c->stream);
  if (e == cudaSuccess) e = tp3::forward(n, rows, true);
  if (e == cudaSuccess) e = tp3::backward(n, rows, d_v, d_w, d_target, shells);
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "mlp backward");
  if (loss) {
    const int nb = rows / 128, nr = d_target ? (rows / shells + 127) / 128 : 0;
    std::vector<double> part(nb), rpart(nr > 0 ? nr : 1);
    int err = 0;
    if ((e = cudaMemcpyAsync(part.data(), n->d_part, nb * sizeof(double), cudaMemcpyDeviceToHost, c->stream)) !=
            cudaSuccess ||
        (nr > 0 && (e = cudaMemcpyAsync(rpart.data(), n->d_part + n->max_rows / 128, nr * sizeof(double),
                                        cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess) ||
        (e = cudaMemcpyAsync(&err, n->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(c->stream)) != cudaSuccess)
      return tp3::ctx_cuda_fail(c, e, "mlp loss read");
    if (err) return tp3::ctx_fail(c, err, "a bounded wait in the mlp GEMM ran out");
    double sum = 0.0;
    for (double p : part) sum += p;
    for (int b = 0; b < nr; ++b) sum += rpart[b];
    *loss = sum;
  }
  return TP3_OK;
}

int tp3_mlp_loss_grad(tp3_mlp* n, int rows, const void* d_x, const float* d_v, const float* d_w,
                      const float* d_target, int shells, double* loss, float* grad_host) {
  if (!n) return TP3_ERR_ARG;
  double l = 0.0;
  if (int r = mlp_loss_grad(n, rows, d_x, d_v, d_w, d_target, shells, &l)) return r;
  if (loss) *loss = l;
  if (grad_host) {
    tp3_ctx* c = n->ctx;
    cudaError_t e = cudaMemcpyAsync(grad_host, n->d_grad, n->n_par * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "mlp grad read");
  }
  return TP3_OK;
}

int tp3_mlp_train_step(tp3_mlp* n, int rows, const void* d_x, const float* d_v, const float* d_w,
                       const float* d_target, int shells, float lr, double* loss) {
  if (!n) return TP3_ERR_ARG;
  if (int r = mlp_loss_grad(n, rows, d_x, d_v, d_w, d_target, shells, loss)) return r;
  tp3_ctx* c = n->ctx;
  n->adam_t += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - (float)std::pow((double)b1, (double)n->adam_t);
  const float c2 = 1.f - (float)std::pow((double)b2, (double)n->adam_t);
  tp3::k_adam<<<(unsigned)((n->n_par + 255) / 256), 256, 0, c->stream>>>(n->d_par, n->d_grad, n->d_m, n->d_v, n->n_par,
                                                                         lr, b1, b2, 1e-8f, c1, c2);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = tp3::pack_all(n);
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "mlp adam");
  return TP3_OK;
}

}  // extern "C"
