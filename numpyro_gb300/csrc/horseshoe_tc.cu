// horseshoe_tc.cu -- tensor-core (tcgen05 + TMA + TMEM) GEMMs of the horseshoe (Gaussian GLM)
// potential, the precision="bf16x3" path of GBN_FAMILY_HORSESHOE.
//
// U needs R = y - X beta for every chain (N rows) and the adjoint X^T R.  Both contractions run as
//   D[128 chains][64 cols] = sum_k A[chain][k] B[col][k]        (both operands K-major, bf16)
// on tcgen05, with each FP32 operand written exactly enough as three bf16 terms (hi + mid + lo,
// 24 significant bits) and the six cross products whose term orders sum to at most 2
// (hh, hm, mh, hl, lh, mm); the dropped products are below 2^-24 of the result.
// The tensor core's FP32 accumulation does not round to nearest, and its bias is coherent across
// rows, which shows up in sum R^2.  So the dominant hh products go to a double-buffered TMEM
// accumulator that the epilogue drains after every 64-wide K block and sums in FP32 registers
// (round to nearest); the five correction products (2^-8 smaller) share one accumulator for the
// whole K range.
//   GEMM1  A = beta splits [3][Cp][Kp], B = X splits [3][Np][Kp]  -> R^T[chain][row] = y - D,
//          written back as bf16 splits (GEMM2's A operand) with per-(row tile, chain) sums of R^2
//   GEMM2  A = R^T splits [3][Cp][Np], B = X^T splits [3][Pp][Np] -> partials of X^T R per
//          row range (split-K), reduced by horseshoe_finish_kernel
// X and X^T are split once per model; beta is split from the chains' positions every tick.
// One CTA: warp 0 TMA producer (3-stage ring of 72 KB), warp 1 MMA issuer, warps 2..5 epilogue
// (one TMEM lane quadrant each).  Every mbarrier wait is bounded; on a timeout the CTA records an
// error, drains its copies and MMAs (bounded), frees TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "tc_ptx.cuh"

namespace gbn {
namespace hstc {
using namespace tc;

constexpr int TM = 128;  // MMA M: chains per tile (TMEM lanes)
constexpr int TN = 64;   // MMA N: rows (GEMM1) or features (GEMM2) per tile
constexpr int TK = 64;   // K per stage: one 128-byte swizzle row of bf16
constexpr int NSPL = 3;  // bf16 terms per operand
constexpr int STAGES = 3;
constexpr int A_SPLIT = TM * TK * 2;                     // 16 KB
constexpr int B_SPLIT = TN * TK * 2;                     // 8 KB
constexpr int STAGE_BYTES = NSPL * (A_SPLIT + B_SPLIT);  // 72 KB
constexpr int OFF_MISC = STAGES * STAGE_BYTES;
constexpr int NUM_BARS = 2 * STAGES + 5;  // full, empty per stage; hh full/empty x 2; done
constexpr int SMEM_BYTES = OFF_MISC + 256 + 1024;  // + alignment slack
constexpr int NUM_THREADS = 32 * 6;
constexpr uint32_t TMEM_COLS = 256;  // hh accumulators at columns 0 and 64, corrections at 128
constexpr uint32_t CORR_COL = 128;
constexpr int NPAIRS = 6;  // (A term, B term): hh, hm, mh, hl, lh, mm

struct GemmArgs {
  int mode;              // 1: residuals (GEMM1), 2: adjoint partials (GEMM2)
  int a_rows_split;      // rows of one split in A's tensor (Cp)
  int b_rows_split;      // rows of one split in B's tensor
  int kblocks;           // K / TK
  int kblocks_per_split; // split-K
  int n_valid;           // valid columns (rows of the data for GEMM1, features for GEMM2)
  // mode 1
  const float* y;
  __nv_bfloat16* rt;  // R^T splits [3][Cp][rt_ld]
  int rt_ld;
  double* part_rr;  // [column tiles][ld_rr]
  int ld_rr;
  int npts;
  // mode 2
  float* part_gb;  // [splits][npts][ldg]
  int ldg;
  int* err;
  const int32_t* pending;
};

// two values -> their hi/mid/lo bf16 terms, each pair packed in one 32-bit word
__device__ __forceinline__ void split3_pair(float a, float b, uint32_t& h, uint32_t& m, uint32_t& l) {
  const __nv_bfloat162 h2 = __floats2bfloat162_rn(a, b);
  const float2 hf = __bfloat1622float2(h2);
  const float ra = a - hf.x, rb = b - hf.y;
  const __nv_bfloat162 m2 = __floats2bfloat162_rn(ra, rb);
  const float2 mf = __bfloat1622float2(m2);
  const __nv_bfloat162 l2 = __floats2bfloat162_rn(ra - mf.x, rb - mf.y);
  h = *reinterpret_cast<const uint32_t*>(&h2);
  m = *reinterpret_cast<const uint32_t*>(&m2);
  l = *reinterpret_cast<const uint32_t*>(&l2);
}
__device__ __forceinline__ void split3(float v, __nv_bfloat16& h, __nv_bfloat16& m, __nv_bfloat16& l) {
  h = __float2bfloat16_rn(v);
  const float r1 = v - __bfloat162float(h);
  m = __float2bfloat16_rn(r1);
  l = __float2bfloat16_rn(r1 - __bfloat162float(m));
}

__global__ void __launch_bounds__(NUM_THREADS, 1) hs_tc_gemm_kernel(const __grid_constant__ CUtensorMap ta,
                                                                    const __grid_constant__ CUtensorMap tb,
                                                                    GemmArgs G) {
  if (G.pending && *G.pending == 0) return;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + OFF_MISC);
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(smem + OFF_MISC + NUM_BARS * 8);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + OFF_MISC + NUM_BARS * 8 + 4);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n0 = blockIdx.x * TN, m0 = blockIdx.y * TM;
  const int kb0 = blockIdx.z * G.kblocks_per_split;
  const int nkb = max(0, min(G.kblocks, kb0 + G.kblocks_per_split) - kb0);
  auto full = [&](int s) { return smem_u32(&bars[s]); };
  auto empty = [&](int s) { return smem_u32(&bars[STAGES + s]); };
  auto hfull = [&](int b) { return smem_u32(&bars[2 * STAGES + b]); };
  auto hempty = [&](int b) { return smem_u32(&bars[2 * STAGES + 2 + b]); };
  const uint32_t done = smem_u32(&bars[2 * STAGES + 4]);

  if (threadIdx.x == 0) {
    for (int i = 0; i < STAGES; ++i) {
      bar_init(full(i), 1);
      bar_init(empty(i), 1);
    }
    for (int b = 0; b < 2; ++b) {
      bar_init(hfull(b), 1);
      bar_init(hempty(b), 4);  // the four epilogue warps
    }
    bar_init(done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_holder)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_holder;

  if (warp == 0) {
    // ------------------------------------------------------------ TMA producer
    if (lane == 0) {
      int issued = 0;
      for (int i = 0; i < nkb; ++i) {
        const int s = i % STAGES;
        if (i >= STAGES && !bar_wait(empty(s), ((i / STAGES) - 1) & 1, abort_flag, G.err)) break;
        const int kx = (kb0 + i) * TK;
        uint8_t* st = smem + s * STAGE_BYTES;
        bar_expect_tx(full(s), STAGE_BYTES);
        for (int sp = 0; sp < NSPL; ++sp) {
          tma_load_2d(smem_u32(st + sp * A_SPLIT), &ta, kx, sp * G.a_rows_split + m0, full(s));
          tma_load_2d(smem_u32(st + NSPL * A_SPLIT + sp * B_SPLIT), &tb, kx, sp * G.b_rows_split + n0, full(s));
        }
        issued = i + 1;
      }
      if (*abort_flag) {  // drain copies still in flight before the CTA can exit
        for (int i = (issued > STAGES ? issued - STAGES : 0); i < issued; ++i) {
          const int s = i % STAGES;
          for (uint32_t k = 0; k < WAIT_LIMIT && !bar_try(full(s), (i / STAGES) & 1); ++k) {
          }
        }
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    // The whole warp runs the loop and one elected lane issues each MMA and commit (issued by
    // lane 0 alone, every tcgen05.mma paid a long issue latency); the stage descriptors are built
    // once and moved by constant offsets.
    constexpr uint32_t ID = idesc(TM, TN, 0, 0);  // both operands K-major
    constexpr int kPairA[NPAIRS] = {0, 0, 1, 0, 2, 1};
    constexpr int kPairB[NPAIRS] = {0, 1, 0, 2, 0, 1};
    const uint64_t d0 = sdesc(smem_u32(smem), 16, 1024);  // stage 0, offset 0
    for (int i = 0; i < nkb; ++i) {
      const int s = i % STAGES, hb = i & 1;
      if (!bar_wait_warp(full(s), (i / STAGES) & 1, abort_flag, G.err)) break;
      if (i >= 2 && !bar_wait_warp(hempty(hb), ((i >> 1) - 1) & 1, abort_flag, G.err)) break;
      tc_fence_after();
      const uint64_t st = sdesc_at(d0, (uint32_t)(s * STAGE_BYTES));
#pragma unroll
      for (int kk = 0; kk < TK / 16; ++kk)  // hh of this block into its own accumulator
        mma_bf16_warp(tmem + (uint32_t)(hb * TN), sdesc_at(st, kk * 32), sdesc_at(st, NSPL * A_SPLIT + kk * 32), ID,
                      kk > 0 ? 1u : 0u);
      mma_commit_warp(hfull(hb));
#pragma unroll
      for (int p = 1; p < NPAIRS; ++p) {  // corrections accumulate over the whole K range
#pragma unroll
        for (int kk = 0; kk < TK / 16; ++kk)
          mma_bf16_warp(tmem + CORR_COL, sdesc_at(st, kPairA[p] * A_SPLIT + kk * 32),
                        sdesc_at(st, NSPL * A_SPLIT + kPairB[p] * B_SPLIT + kk * 32), ID,
                        (i > 0 || p > 1 || kk > 0) ? 1u : 0u);
      }
      mma_commit_warp(empty(s));
    }
    __syncwarp();
    mma_commit_warp(done);
    // every MMA issued by this warp has completed before TMEM can be released
    for (uint32_t k = 0; k < WAIT_LIMIT && !bar_try(done, 0); ++k) {
    }
  } else {
    // ------------------------------------------------------------ epilogue (warps 2..5)
    const int q = warp & 3;
    const int chain = m0 + q * 32 + lane;  // TMEM lane = chain
    const uint32_t lrow = (uint32_t)(q * 32) << 16;
    float acc[TN];
#pragma unroll
    for (int e = 0; e < TN; ++e) acc[e] = 0.0f;
    bool ok = true;
    for (int i = 0; i < nkb && ok; ++i) {  // drain each block's hh accumulator, round-to-nearest sums
      const int hb = i & 1;
      ok = bar_wait(hfull(hb), (i >> 1) & 1, abort_flag, G.err);
      if (!ok) break;
      tc_fence_after();
#pragma unroll
      for (int j = 0; j < TN / 16; ++j) {
        float v[16];
        tmem_ld16(tmem + lrow + (uint32_t)(hb * TN + 16 * j), v);
        tmem_wait_ld();
#pragma unroll
        for (int e = 0; e < 16; ++e) acc[16 * j + e] += v[e];
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) bar_arrive(hempty(hb));
    }
    if (ok) ok = bar_wait(done, 0, abort_flag, G.err);
    if (ok) {
      tc_fence_after();
      double rr = 0.0;
#pragma unroll
      for (int j = 0; j < TN / 16; ++j) {
        float v[16];
        if (nkb > 0) {
          tmem_ld16(tmem + lrow + CORR_COL + (uint32_t)(16 * j), v);
          tmem_wait_ld();
        } else {
#pragma unroll
          for (int e = 0; e < 16; ++e) v[e] = 0.0f;
        }
#pragma unroll
        for (int e = 0; e < 16; ++e) v[e] += acc[16 * j + e];
        const int c0 = n0 + 16 * j;
        if (G.mode == 1) {
          // R = y - X beta for rows c0..c0+15 (zero past the data) and its bf16 terms
          uint32_t hw[8], mw[8], lw[8];
          float sq = 0.0f;
#pragma unroll
          for (int e = 0; e < 16; e += 2) {
            const float ra = (c0 + e < G.n_valid) ? G.y[c0 + e] - v[e] : 0.0f;
            const float rb = (c0 + e + 1 < G.n_valid) ? G.y[c0 + e + 1] - v[e + 1] : 0.0f;
            sq = fmaf(ra, ra, sq);
            sq = fmaf(rb, rb, sq);
            split3_pair(ra, rb, hw[e >> 1], mw[e >> 1], lw[e >> 1]);
          }
          rr += (double)sq;
          const size_t o = (size_t)chain * G.rt_ld + c0;
          const size_t sstride = (size_t)G.a_rows_split * G.rt_ld;  // Cp rows per split
          uint4* dh = reinterpret_cast<uint4*>(G.rt + o);
          uint4* dm = reinterpret_cast<uint4*>(G.rt + sstride + o);
          uint4* dl = reinterpret_cast<uint4*>(G.rt + 2 * sstride + o);
          dh[0] = make_uint4(hw[0], hw[1], hw[2], hw[3]);
          dh[1] = make_uint4(hw[4], hw[5], hw[6], hw[7]);
          dm[0] = make_uint4(mw[0], mw[1], mw[2], mw[3]);
          dm[1] = make_uint4(mw[4], mw[5], mw[6], mw[7]);
          dl[0] = make_uint4(lw[0], lw[1], lw[2], lw[3]);
          dl[1] = make_uint4(lw[4], lw[5], lw[6], lw[7]);
        } else if (chain < G.npts) {
          float* dst = G.part_gb + ((size_t)blockIdx.z * G.npts + chain) * G.ldg + c0;
#pragma unroll
          for (int e = 0; e < 16; e += 4)
            if (c0 + e < G.ldg) *reinterpret_cast<float4*>(dst + e) = make_float4(v[e], v[e + 1], v[e + 2], v[e + 3]);
        }
      }
      if (G.mode == 1 && chain < G.npts) G.part_rr[(size_t)blockIdx.x * G.ld_rr + chain] = rr;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// X [n][p] fp32 -> splits [3][rows][ld] bf16 (transposed: X^T [p][n]); zero padding
__global__ void split_matrix_kernel(const float* __restrict__ x, int64_t n, int p, int transpose, int rows, int ld,
                                    __nv_bfloat16* __restrict__ out) {
  const int64_t total = (int64_t)rows * ld;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / ld, k = i % ld;
    float v = 0.0f;
    if (!transpose && r < n && k < p) v = x[r * p + k];
    if (transpose && r < p && k < n) v = x[k * p + r];
    __nv_bfloat16 h, m, l;
    split3(v, h, m, l);
    out[i] = h;
    out[total + i] = m;
    out[2 * total + i] = l;
  }
}

// beta [npts] rows (centred: z[0:P]; non-centred: exp(log tau + log lambda) * unscaled) -> splits
// [3][Cp][Kp] bf16, zero padding
__global__ void split_beta_kernel(const float* __restrict__ Q, int npts, int ld, int P, int noncentred, int cp,
                                  int kp, __nv_bfloat16* __restrict__ out, const int32_t* pending) {
  if (pending && *pending == 0) return;
  const int64_t total = (int64_t)cp * kp;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i / kp), k = (int)(i % kp);
    float v = 0.0f;
    if (c < npts && k < P) {
      const float* z = Q + (size_t)c * ld;
      v = noncentred ? expf(z[P + 1] + z[k]) * z[P + 2 + k] : z[k];
    }
    __nv_bfloat16 h, m, l;
    split3(v, h, m, l);
    out[i] = h;
    out[total + i] = m;
    out[2 * total + i] = l;
  }
}

struct HsState {
  int np = 0, kp = 0, pp = 0, cp = 0, splits = 4;
  __nv_bfloat16 *xs = nullptr, *xts = nullptr, *bs = nullptr, *rts = nullptr;
  float* part_gb = nullptr;
  double* part_rr = nullptr;
  int* err = nullptr;
  CUtensorMap tm_x, tm_xt, tm_b, tm_rt;
  bool ok = false;
};

}  // namespace hstc

static PFN_cuTensorMapEncodeTiled_v12000 hs_get_encode() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// bf16 splits [3 * rows][ld] as a 2-D tensor map with box {64, box_rows}, 128-byte swizzle
static bool hs_encode(CUtensorMap* map, void* base, int ld, int total_rows, int box_rows) {
  cuuint64_t gdim[2] = {(cuuint64_t)ld, (cuuint64_t)total_rows};
  cuuint64_t gstride[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {(cuuint32_t)hstc::TK, (cuuint32_t)box_rows};
  cuuint32_t estride[2] = {1, 1};
  return hs_get_encode()(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, gdim, gstride, box, estride,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

static int round_up(int v, int m) { return (v + m - 1) / m * m; }

bool horseshoe_tc_supported(const ModelDev& m) {
  if (m.family != 3 || m.n <= 0 || m.n >= (int64_t)1 << 30) return false;
  int dev = 0, major = 0, minor = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  return major == 10 && minor == 3 && hs_get_encode() != nullptr;
}

cudaError_t horseshoe_tc_prepare(ModelDev& m, int points) {
  using namespace hstc;
  HsState* s = reinterpret_cast<HsState*>(m.hs_tc);
  cudaError_t e = cudaSuccess;
  if (!s) {
    s = new HsState();
    m.hs_tc = s;
    s->np = round_up((int)m.n, TK);   // data rows: GEMM1 column tiles, GEMM2 K
    s->kp = round_up(m.p, TK);        // features as GEMM1 K
    s->pp = round_up(m.p, TN);        // features as GEMM2 columns
    s->cp = round_up(points, TM);
    const size_t nx = 3 * (size_t)s->np * s->kp, nxt = 3 * (size_t)s->pp * s->np;
    e = cudaMalloc(&s->xs, sizeof(__nv_bfloat16) * nx);
    if (e == cudaSuccess) e = cudaMalloc(&s->xts, sizeof(__nv_bfloat16) * nxt);
    if (e == cudaSuccess) e = cudaMalloc(&s->bs, sizeof(__nv_bfloat16) * 3 * (size_t)s->cp * s->kp);
    // padding (features k >= p, points c >= npts) stays zero: the fused tick writes only real entries
    if (e == cudaSuccess) e = cudaMemset(s->bs, 0, sizeof(__nv_bfloat16) * 3 * (size_t)s->cp * s->kp);
    if (e == cudaSuccess) e = cudaMalloc(&s->rts, sizeof(__nv_bfloat16) * 3 * (size_t)s->cp * s->np);
    if (e == cudaSuccess) e = cudaMalloc(&s->part_gb, sizeof(float) * (size_t)s->splits * s->cp * s->pp);
    if (e == cudaSuccess) e = cudaMalloc(&s->part_rr, sizeof(double) * (size_t)(s->np / TN) * s->cp);
    if (e == cudaSuccess) e = cudaMalloc(&s->err, sizeof(int));
    if (e != cudaSuccess) return e;
    cudaMemset(s->err, 0, sizeof(int));
    split_matrix_kernel<<<1024, 256>>>(m.x, m.n, m.p, 0, s->np, s->kp, s->xs);
    split_matrix_kernel<<<1024, 256>>>(m.x, m.n, m.p, 1, s->pp, s->np, s->xts);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    bool ok = hs_encode(&s->tm_x, s->xs, s->kp, 3 * s->np, TN) && hs_encode(&s->tm_xt, s->xts, s->np, 3 * s->pp, TN) &&
              hs_encode(&s->tm_b, s->bs, s->kp, 3 * s->cp, TM) && hs_encode(&s->tm_rt, s->rts, s->np, 3 * s->cp, TM);
    if (!ok) return cudaErrorInvalidValue;
    e = cudaFuncSetAttribute(hs_tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return e;
    s->ok = true;
  }
  if (round_up(points, TM) > s->cp) return cudaErrorInvalidValue;  // sized for the handle's chains
  return e;
}

void horseshoe_tc_free(ModelDev& m) {
  hstc::HsState* s = reinterpret_cast<hstc::HsState*>(m.hs_tc);
  if (!s) return;
  cudaFree(s->xs);
  cudaFree(s->xts);
  cudaFree(s->bs);
  cudaFree(s->rts);
  cudaFree(s->part_gb);
  cudaFree(s->part_rr);
  cudaFree(s->err);
  delete s;
  m.hs_tc = nullptr;
}

int* horseshoe_tc_error_ptr(const ModelDev& m) {
  hstc::HsState* s = reinterpret_cast<hstc::HsState*>(m.hs_tc);
  return s ? s->err : nullptr;
}

int horseshoe_tc_error(const ModelDev& m) {
  hstc::HsState* s = reinterpret_cast<hstc::HsState*>(m.hs_tc);
  if (!s) return 0;
  int v = 0;
  cudaMemcpy(&v, s->err, sizeof(int), cudaMemcpyDeviceToHost);
  return v;
}

void horseshoe_finish_launch(const float* Q, int npts, int ld, int P, int64_t N, const float* part_gb, int splits,
                             int ldg, const double* part_rr, int ld_rr, int mtiles, int noncentred, double* PE,
                             float* G, const int32_t* pending, cudaStream_t st);

bool horseshoe_tc_fusion(ModelDev& m, int npts, AdvParams* P) {
  using namespace hstc;
  if (horseshoe_tc_prepare(m, npts) != cudaSuccess) return false;
  HsState* s = reinterpret_cast<HsState*>(m.hs_tc);
  if (!s || !s->ok) return false;
  P->hsf_part_gb = s->part_gb;
  P->hsf_part_rr = s->part_rr;
  P->hsf_bs = reinterpret_cast<uint16_t*>(s->bs);
  P->hsf_N = m.n;
  P->hsf_total = (int64_t)s->cp * s->kp;
  P->hsf_P = m.p;
  P->hsf_kp = s->kp;
  P->hsf_splits = s->splits;
  P->hsf_ldg = s->pp;
  P->hsf_ld_rr = s->cp;
  P->hsf_mtiles = s->np / TN;
  P->hsf_nc = m.hyper[0] != 0.0;
  return true;
}

cudaError_t horseshoe_tc_launch(ModelDev& m, const float* Q, int npts, double* PE, float* G, const int32_t* pending,
                                cudaStream_t st, bool fused_tick) {
  using namespace hstc;
  HsState* s = reinterpret_cast<HsState*>(m.hs_tc);
  if (!s || !s->ok) return cudaErrorNotSupported;
  cudaError_t e = horseshoe_tc_prepare(m, npts);
  if (e != cudaSuccess) return e;
  const int cp = round_up(npts, TM), nc = m.hyper[0] != 0.0;
  // In the tick engine's fused form the state-machine kernel writes the coefficient terms with the
  // positions and finishes the potential, so only the two GEMMs run here.
  if (!fused_tick)
    split_beta_kernel<<<std::min(1024, (cp * s->kp + 255) / 256), 256, 0, st>>>(Q, npts, m.D, m.p, nc, s->cp, s->kp,
                                                                                 s->bs, pending);
  GemmArgs g1{};
  g1.mode = 1;
  g1.a_rows_split = s->cp;
  g1.b_rows_split = s->np;
  g1.kblocks = s->kp / TK;
  g1.kblocks_per_split = g1.kblocks;
  g1.n_valid = (int)m.n;
  g1.y = m.y;
  g1.rt = s->rts;
  g1.rt_ld = s->np;
  g1.part_rr = s->part_rr;
  g1.ld_rr = s->cp;
  g1.npts = npts;
  g1.err = s->err;
  g1.pending = pending;
  hs_tc_gemm_kernel<<<dim3(s->np / TN, cp / TM, 1), NUM_THREADS, SMEM_BYTES, st>>>(s->tm_b, s->tm_x, g1);
  GemmArgs g2{};
  g2.mode = 2;
  g2.a_rows_split = s->cp;
  g2.b_rows_split = s->pp;
  g2.kblocks = s->np / TK;
  g2.kblocks_per_split = (g2.kblocks + s->splits - 1) / s->splits;
  g2.n_valid = m.p;
  g2.npts = npts;
  g2.part_gb = s->part_gb;
  g2.ldg = s->pp;
  g2.err = s->err;
  g2.pending = pending;
  hs_tc_gemm_kernel<<<dim3(s->pp / TN, cp / TM, s->splits), NUM_THREADS, SMEM_BYTES, st>>>(s->tm_rt, s->tm_xt, g2);
  if (!fused_tick)
    horseshoe_finish_launch(Q, npts, m.D, m.p, m.n, s->part_gb, s->splits, s->pp, s->part_rr, s->cp, s->np / TN, nc,
                            PE, G, pending, st);
  return cudaGetLastError();
}

}  // namespace gbn
