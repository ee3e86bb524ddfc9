// logreg_tc.cu -- tensor-core (tcgen05 + TMA + TMEM) logistic-regression potential.
//
// U(b) = sum_n [softplus(l_n) - y_n l_n] + sum_d b_d^2 / (2 s^2) + const,  l = X b
// dU/db = X^T (sigmoid(l) - y) + b / s^2
// (numpyro: BernoulliLogits.log_prob discrete.py:263 via
//  binary_cross_entropy_with_logits distributions/util.py:317-320, Normal prior
//  continuous.py:2975-2989, potential_energy infer/util.py:333-358.)
//
// Sign-flipped rows.  With s_n = 1 - 2 y_n and X'_n = s_n X_n (exact in bf16):
//   softplus(l_n) - y_n l_n = softplus(l'_n) = l'_n/2 + |l'_n|/2 + log(1 + e^{-|l'_n|}),  l' = X' b
//   sum_n (sigmoid(l_n) - y_n) X_n = sum_n sigmoid(l'_n) X'_n
// so the kernel never reads y: it streams X' and the linear part sum_n l'_n / 2 = (X'^T 1 / 2) . b
// is added per chain from a vector computed once.
//
// One CTA owns 128 chains and a strided set of 128-row tiles of X':
//   warp 0      TMA producer: X' tile [128 rows x 64 feat] bf16, 128B swizzle, 4-stage ring
//   warp 1      MMA issuer:  GEMM1  H[128 chains x 128 rows] = (b_hi + b_mid + b_lo)/2 . X'_tile^T
//                            (three K=64 BF16 products accumulate in FP32 in TMEM, so the
//                            FP32 coefficients are represented exactly: "bf16x3"),
//                            GEMM2  G[128 chains x 64 feat] += E . X'_tile  (E = sigmoid(l'))
//   warps 2..17 epilogue: TMEM lanes are chains, columns rows.  Two groups of 8 warps take
//               alternate tiles (one H buffer each); in a group 2 warps per lane quadrant split
//               the 128 rows.  Per logit one ex2 and one tanh; log(1 + e^{-|l'|}) is taken as one
//               lg2 of the product of 8 rows' factors (2.125 special-function ops per logit).
//               E goes to shared memory as bf16 in the K-major layout GEMM2 reads.  Each thread
//               accumulates its chain's log-likelihood over its rows; the four threads of a
//               chain are combined once per CTA in FP64.
// H is double-buffered in TMEM (2 x 128 columns) so GEMM1 of tile t+1 overlaps the
// epilogue of tile t; G lives in TMEM for the whole launch (64 columns).
// The design matrix must be exactly representable in bf16 (checked on the host).
// Every mbarrier wait is bounded; on a timeout the CTA records an error, drains its
// in-flight copies and MMAs (bounded), frees TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <cstdio>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "tc_ptx.cuh"

namespace gbn {
namespace tc {

constexpr int BM = 128;  // rows per tile
constexpr int BN = 128;  // chains per CTA
constexpr int BK = 64;   // padded features: one 128-byte swizzle row of bf16
constexpr int NSPLIT = 3;
constexpr int STAGES = 4;
constexpr int X_TILE = BM * BK * 2;  // 16 KB
constexpr int B_TILE = BN * BK * 2;  // 16 KB
constexpr int S_TILE = BM * BN * 2;  // 32 KB
constexpr int OFF_X = 0;
constexpr int OFF_B = OFF_X + STAGES * X_TILE;
constexpr int OFF_S = OFF_B + NSPLIT * B_TILE;
constexpr int OFF_MISC = OFF_S + 2 * S_TILE;
constexpr int NUM_BARS = 2 * STAGES + 2 + 2 + 2 + 2 + 1;
constexpr int SMEM_BYTES = OFF_MISC + 256 + BN * 8 + 1024;  // + alignment slack
constexpr int EPI_WARPS = 16;             // epilogue warps: 4 per TMEM lane quadrant
constexpr int EPI_GROUP = EPI_WARPS / 2;  // warps that share one tile (one accumulator buffer)
constexpr int GCOLS = BK * 4 / EPI_WARPS; // gradient columns read back per epilogue warp
constexpr int NUM_THREADS = 32 * (2 + EPI_WARPS);
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t ACC2_COL = 256;

enum { B_XFULL = 0, B_XEMPTY = STAGES, B_ACCF = 2 * STAGES, B_ACCE = 2 * STAGES + 2, B_SF = 2 * STAGES + 4,
       B_SE = 2 * STAGES + 6, B_DONE = 2 * STAGES + 8 };

// One tile of the epilogue for one warp: its lane's chain x 32 rows (TMEM columns at taddr).
// TMEM holds h = l'/2 (the coefficients enter GEMM1 halved, an exact scaling).  Per row:
//   E = sigmoid(l') = tanh(h)/2 + 1/2                      -> bf16, K-major tile for GEMM2
//       (forming it by Newton's method on the FMA pipe for half the rows measured slower:
//       with 2.125 special-function ops per logit the epilogue is issue-bound)
//   softplus(l') - l'/2 = |h| + log(1 + e^{-2|h|})          -> |h| summed, the logs taken as
//                                                            one log2 per product of 8 rows
// With MASK, rows r >= nvalid lie past the end of the data: they are left out of the
// log-likelihood (their X' rows are zero, so E needs no mask).
// E is written to erow: this chain's 128-byte row of the swizzled K-major tile, 16-byte chunk
// chunk0 + g for rows 8g..8g+7, XOR-swizzled with the chain index cx = chain & 7.
// With release, this warp's last read of the accumulator buffer is signalled on acc_empty_bar.
template <bool MASK>
__device__ __forceinline__ void epilogue_tile(uint32_t taddr, uint8_t* erow, int chunk0, int cx, int nvalid,
                                              float& sabs, float& slg, bool release, uint32_t acc_empty_bar,
                                              int lane) {
  const float NEG_2LOG2E = -2.8853900817779268f;
  uint32_t v[2][16];
  tmem_ld16u(taddr, v[0]);
  tmem_ld16u(taddr + 16, v[1]);
  tmem_wait16(v[0]);
  tmem_wait16(v[1]);
  if (release) {  // every column of this warp's share has been read: release the accumulator
    tc_fence_before();
    __syncwarp();
    if (lane == 0) bar_arrive(acc_empty_bar);
  }
  float ta = 0.0f, tl = 0.0f;
#pragma unroll
  for (int g8 = 0; g8 < 4; ++g8) {
    float prod = 1.0f;
    uint32_t pk[4];
#pragma unroll
    for (int e = 0; e < 8; e += 2) {
      float ev[2];
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        const int r = 8 * g8 + e + hh;
        const float h = __uint_as_float(v[r >> 4][r & 15]);
        const float t = ex2_approx(fabsf(h) * NEG_2LOG2E);  // e^{-|l'|}
        if (!MASK || r < nvalid) {
          ta += fabsf(h);
          prod = fmaf(prod, t, prod);  // prod * (1 + t), one rounding
        }
        ev[hh] = fmaf(0.5f, tanh_approx(h), 0.5f);
      }
      pk[e >> 1] = pack_bf16(ev[0], ev[1]);
    }
    tl += lg2_approx(prod);
    *reinterpret_cast<uint4*>(erow + (((chunk0 + g8) ^ cx) << 4)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
  }
  sabs += ta;
  slg += tl;
}

struct Params {
  int64_t n;
  const __nv_bfloat16* bsplit;  // [chain_blocks*128][3][64]
  int npts;
  int row_groups;
  float* part_g;    // [row_groups][npts][64]
  double* part_ll;  // [row_groups][npts]
  int* err;
  const int32_t* pending;
};

__global__ void __launch_bounds__(NUM_THREADS, 1) logreg_tc_kernel(const __grid_constant__ CUtensorMap tmap_x,
                                                                   Params P) {
  if (P.pending && *P.pending == 0) return;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + OFF_MISC);
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(smem + OFF_MISC + NUM_BARS * 8);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + OFF_MISC + NUM_BARS * 8 + 4);
  double* ll_smem = reinterpret_cast<double*>(smem + OFF_MISC + 256);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cb = blockIdx.x;  // chain block
  const int rg = blockIdx.y;  // row group
  const int64_t ntiles = (P.n + BM - 1) / BM;
  const int my_tiles = (int)((ntiles - rg + P.row_groups - 1) / P.row_groups);
  auto bar = [&](int i) { return smem_u32(&bars[i]); };

  if (threadIdx.x == 0) {
    for (int i = 0; i < STAGES; ++i) {
      bar_init(bar(B_XFULL + i), 1);
      bar_init(bar(B_XEMPTY + i), 1);
    }
    for (int i = 0; i < 2; ++i) {
      bar_init(bar(B_ACCF + i), 1);
      bar_init(bar(B_ACCE + i), EPI_GROUP);
      bar_init(bar(B_SF + i), EPI_GROUP);
      bar_init(bar(B_SE + i), 1);
    }
    bar_init(bar(B_DONE), 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int i = threadIdx.x; i < BN; i += NUM_THREADS) ll_smem[i] = 0.0;
  // coefficient splits -> K-major 128B-swizzled tiles [128 chains][64 feat] (one per split)
  {
    const uint4* src = reinterpret_cast<const uint4*>(P.bsplit + (size_t)cb * BN * NSPLIT * BK);
    for (int i = threadIdx.x; i < BN * NSPLIT * (BK / 8); i += NUM_THREADS) {
      int chunk = i % (BK / 8);
      int k = (i / (BK / 8)) % NSPLIT;
      int c = i / (NSPLIT * (BK / 8));
      uint4 v = src[i];
      uint32_t off = OFF_B + k * B_TILE + (c >> 3) * 1024 + (c & 7) * 128 + ((chunk ^ (c & 7)) << 4);
      *reinterpret_cast<uint4*>(smem + off) = v;
    }
  }
  fence_proxy_async();
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
      for (int i = 0; i < my_tiles; ++i) {
        int s = i % STAGES;
        if (i >= STAGES && !bar_wait(bar(B_XEMPTY + s), ((i / STAGES) - 1) & 1, abort_flag, P.err)) break;
        int64_t row0 = ((int64_t)rg + (int64_t)i * P.row_groups) * BM;
        bar_expect_tx(bar(B_XFULL + s), X_TILE);
        tma_load_2d(smem_u32(smem + OFF_X + s * X_TILE), &tmap_x, 0, (int)row0, bar(B_XFULL + s));
        issued = i + 1;
      }
      if (*abort_flag) {  // drain copies still in flight before the CTA can exit
        for (int i = (issued > STAGES ? issued - STAGES : 0); i < issued; ++i) {
          int s = i % STAGES;
          for (uint32_t k = 0; k < WAIT_LIMIT && !bar_try(bar(B_XFULL + s), (i / STAGES) & 1); ++k) {
          }
        }
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    // The whole warp runs this loop and one elected lane issues each MMA and commit: from a
    // converged warp the descriptor arithmetic stays warp-uniform.  (Run by lane 0 alone,
    // each tcgen05.mma took ~70-90 cycles to issue and this loop, not the tensor pipe or the
    // epilogue, set the tile rate.)  Descriptors are built once and moved by constant offsets.
    constexpr uint32_t ID1 = idesc(BN, BM, 0, 0);  // H = B . X'^T: chains x rows, both K-major
    constexpr uint32_t ID2 = idesc(BN, BK, 0, 1);  // G = E . X': E K-major, X' MN-major
    const uint32_t xb = smem_u32(smem + OFF_X), bb = smem_u32(smem + OFF_B), sb = smem_u32(smem + OFF_S);
    const uint64_t dcoef = sdesc(bb, 16, 1024);  // GEMM1 A: the coefficient splits, the same every tile
    const uint64_t dx1 = sdesc(xb, 16, 1024);    // GEMM1 B: X' tile, K-major, stage 0
    const uint64_t dx2 = sdesc(xb, 1024, 1024);  // GEMM2 B: X' tile, MN-major, stage 0
    const uint64_t de = sdesc(sb, 16, 1024);     // GEMM2 A: E tile, K-major, buffer 0
    bool ok = true;
    for (int i = 0; i <= my_tiles && ok; ++i) {
      if (i < my_tiles) {
        int s = i % STAGES, b = i & 1;
        ok = bar_wait_warp(bar(B_XFULL + s), (i / STAGES) & 1, abort_flag, P.err);
        if (ok && i >= 2) ok = bar_wait_warp(bar(B_ACCE + b), ((i >> 1) - 1) & 1, abort_flag, P.err);
        if (!ok) break;
        tc_fence_after();
        const uint32_t d = tmem + (uint32_t)(b * BN);
        const uint64_t xs = sdesc_at(dx1, (uint32_t)(s * X_TILE));
#pragma unroll
        for (int k = 0; k < NSPLIT; ++k) {
#pragma unroll
          for (int kk = 0; kk < BK / 16; ++kk)
            mma_bf16_warp(d, sdesc_at(dcoef, k * B_TILE + kk * 32), sdesc_at(xs, kk * 32), ID1,
                          (k | kk) ? 1u : 0u);
        }
        mma_commit_warp(bar(B_ACCF + b));
      }
      if (i >= 1) {
        int j = i - 1, s = j % STAGES, b = j & 1;
        ok = bar_wait_warp(bar(B_SF + b), (j >> 1) & 1, abort_flag, P.err);
        if (!ok) break;
        tc_fence_after();
        const uint64_t eb = sdesc_at(de, (uint32_t)(b * S_TILE)), xs = sdesc_at(dx2, (uint32_t)(s * X_TILE));
#pragma unroll
        for (int kk = 0; kk < BM / 16; ++kk) {
          // A = E[b]: K-major [128 chains][128 rows] as two 64-row swizzled halves of 16 KB
          // B = X tile: MN-major (features contiguous), 8-row groups 1024 B apart (SBO)
          mma_bf16_warp(tmem + ACC2_COL, sdesc_at(eb, (kk >> 2) * (BN * 64 * 2) + (kk & 3) * 32),
                        sdesc_at(xs, kk * 2048), ID2, (j > 0 || kk > 0) ? 1u : 0u);
        }
        mma_commit_warp(bar(B_SE + b));
        mma_commit_warp(bar(B_XEMPTY + s));
      }
    }
    __syncwarp();
    mma_commit_warp(bar(B_DONE));
    // wait for every MMA issued by this warp before TMEM can be released
    for (uint32_t k = 0; k < WAIT_LIMIT && !bar_try(bar(B_DONE), 0); ++k) {
    }
  } else {
    // ------------------------------------------------------------ epilogue (warps 2..17)
    // Two groups of 8 warps take alternate tiles, each group one accumulator buffer, so that
    // the groups' TMEM loads and special-function bursts interleave instead of coinciding.
    // In a group, 2 warps per TMEM lane quadrant each take a 64-row half of the tile, as two
    // 32-row parts.
    const int ew = warp - 2;
    const int q = warp & 3;          // TMEM lane quadrant this warp may access: chains 32q..32q+31
    const int grp = ew / EPI_GROUP;  // tiles i with i % 2 == grp, accumulator buffer grp
    const int rh = (ew >> 2) & 1;    // row half of each tile: rows 64 rh .. 64 rh + 63
    const int c = q * 32 + lane;     // this thread's chain within the CTA
    const uint32_t tl = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(grp * BM + rh * 64);
    // this chain's row of the group's E tile (K-major, the 64-row swizzled half rh)
    uint8_t* erow = smem + OFF_S + grp * S_TILE + rh * (BN * 64 * 2) + (c >> 3) * 1024 + (c & 7) * 128;
    Comp32 ll{0.0f, 0.0f};  // log-likelihood of this chain over this thread's rows, all tiles
    bool ok = true;
    for (int i = grp; i < my_tiles && ok; i += 2) {
      const int64_t row0 = ((int64_t)rg + (int64_t)i * P.row_groups) * BM + rh * 64;
      ok = bar_wait(bar(B_ACCF + grp), (i >> 1) & 1, abort_flag, P.err);
      if (ok && i >= 2) ok = bar_wait(bar(B_SE + grp), ((i >> 1) - 1) & 1, abort_flag, P.err);
      if (!ok) break;
      tc_fence_after();
#pragma unroll
      for (int part = 0; part < 2; ++part) {
        float sabs = 0.0f, slg = 0.0f;
        const int64_t nleft = P.n - (row0 + part * 32);
        if (nleft >= 32)
          epilogue_tile<false>(tl + (uint32_t)(part * 32), erow, part * 4, c & 7, 32, sabs, slg, part == 1,
                               bar(B_ACCE + grp), lane);
        else
          epilogue_tile<true>(tl + (uint32_t)(part * 32), erow, part * 4, c & 7, nleft > 0 ? (int)nleft : 0,
                              sabs, slg, part == 1, bar(B_ACCE + grp), lane);
        ll.add(fmaf(0.6931471805599453f, slg, sabs));
      }
      fence_proxy_async();
      __syncwarp();
      if (lane == 0) bar_arrive(bar(B_SF + grp));
    }
    // per-chain sums over the CTA's rows: the chain's four threads meet in shared memory (FP64)
    if (ok) atomicAdd(&ll_smem[c], comp_total(ll));
    // gradient partials: G (lanes = chains, 64 feature columns)
    if (ok) ok = bar_wait(bar(B_DONE), 0, abort_flag, P.err);
    if (ok) {
      tc_fence_after();
      const int gc = cb * BN + c;
#pragma unroll
      for (int j = 0; j < GCOLS / 16; ++j) {
        float v[16];
        const int colb = (ew >> 2) * GCOLS + j * 16;  // 4 warps per lane quadrant split the 64 columns
        tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + ACC2_COL + (uint32_t)colb, v);
        tmem_wait_ld();
        if (gc < P.npts) {
          float4* dst = reinterpret_cast<float4*>(P.part_g + ((size_t)rg * P.npts + gc) * 64 + colb);
#pragma unroll
          for (int k = 0; k < 4; ++k) dst[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (!*abort_flag) {
    for (int i = threadIdx.x; i < BN; i += NUM_THREADS) {
      const int gc = cb * BN + i;
      if (gc < P.npts) P.part_ll[(size_t)rg * P.npts + gc] = ll_smem[i];
    }
  }
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// b (fp32, [npts][ld]) -> [blocks*128][3][64] bf16 with b = hi + mid + lo exactly
__global__ void split_coefs_kernel(const float* __restrict__ Q, int npts, int ld, int p, int npad,
                                   __nv_bfloat16* __restrict__ out, const int32_t* pending) {
  if (pending && *pending == 0) return;
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= npad * BK) return;
  int c = idx / BK, d = idx % BK;
  float v = (c < npts && d < p) ? 0.5f * Q[(size_t)c * ld + d] : 0.0f;  // halved: the kernel works with l/2
  __nv_bfloat16 hi = __float2bfloat16_rn(v);
  float r1 = v - __bfloat162float(hi);
  __nv_bfloat16 mid = __float2bfloat16_rn(r1);
  float r2 = r1 - __bfloat162float(mid);
  __nv_bfloat16 lo = __float2bfloat16_rn(r2);
  __nv_bfloat16* o = out + ((size_t)c * NSPLIT) * BK + d;
  o[0] = hi;
  o[BK] = mid;
  o[2 * BK] = lo;
}

// X'[r] = (1 - 2 y_r) X[r] in bf16, rows padded to 64 features; flags values bf16 cannot hold
__global__ void to_bf16_kernel(const float* __restrict__ x, const float* __restrict__ y, int64_t n, int p,
                               __nv_bfloat16* __restrict__ out, int* inexact) {
  int64_t total = n * BK;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = i / BK;
    int d = (int)(i % BK);
    const float sgn = (y[r] > 0.5f) ? -1.0f : 1.0f;
    float v = (d < p) ? sgn * x[r * p + d] : 0.0f;
    __nv_bfloat16 h = __float2bfloat16_rn(v);
    if (__bfloat162float(h) != v) atomicExch(inexact, 1);
    out[i] = h;
  }
}

// lin[d] = sum_r (1/2 - y_r) X_rd = (X'^T 1 / 2)_d in FP64 (the linear part of the log-likelihood)
__global__ void linear_term_kernel(const float* __restrict__ x, const float* __restrict__ y, int64_t n, int p,
                                   double* __restrict__ lin) {
  __shared__ double part[4][64];
  const int d = threadIdx.x & 63, rl = threadIdx.x >> 6;
  double s = 0.0;
  if (d < p)
    for (int64_t r = (int64_t)blockIdx.x * 4 + rl; r < n; r += (int64_t)gridDim.x * 4)
      s += (0.5 - (double)y[r]) * (double)x[r * p + d];
  part[rl][d] = s;
  __syncthreads();
  if (rl == 0 && d < p) atomicAdd(&lin[d], part[0][d] + part[1][d] + part[2][d] + part[3][d]);
}

struct TCState {
  double* lin = nullptr;
  __nv_bfloat16* xb = nullptr;
  __nv_bfloat16* bsplit = nullptr;
  CUtensorMap tmap;
  int* err = nullptr;
  int bsplit_pts = 0;
  int row_groups = 0;
  int chain_blocks = 0;
  bool ok = false;
};

}  // namespace tc

static PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
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

bool logreg_tc_supported(const ModelDev& m) {
  if (m.family != 2 || m.p > tc::BK || m.n <= 0 || m.n >= (int64_t)1 << 31) return false;
  int dev = 0, major = 0, minor = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  if (major != 10 || minor != 3) return false;
  return get_encode() != nullptr;
}

cudaError_t logreg_tc_prepare(ModelDev& m, int points) {
  tc::TCState* s = reinterpret_cast<tc::TCState*>(m.tc);
  cudaError_t e = cudaSuccess;
  if (!s) {
    s = new tc::TCState();
    m.tc = s;
    e = cudaMalloc(&s->xb, sizeof(__nv_bfloat16) * (size_t)m.n * tc::BK);
    if (e == cudaSuccess) e = cudaMalloc(&s->err, sizeof(int) * 2);
    if (e != cudaSuccess) return e;
    cudaMemset(s->err, 0, sizeof(int) * 2);
    tc::to_bf16_kernel<<<1024, 256>>>(m.x, m.y, m.n, m.p, s->xb, s->err + 1);
    int inexact = 0;
    e = cudaMemcpy(&inexact, s->err + 1, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return e;
    if (inexact) return cudaErrorNotSupported;  // design matrix not exactly representable in bf16
    e = cudaMalloc(&s->lin, sizeof(double) * tc::BK);
    if (e != cudaSuccess) return e;
    cudaMemset(s->lin, 0, sizeof(double) * tc::BK);
    tc::linear_term_kernel<<<1024, 256>>>(m.x, m.y, m.n, m.p, s->lin);
    cuuint64_t gdim[2] = {(cuuint64_t)tc::BK, (cuuint64_t)m.n};
    cuuint64_t gstride[1] = {(cuuint64_t)tc::BK * 2};
    cuuint32_t box[2] = {(cuuint32_t)tc::BK, (cuuint32_t)tc::BM};
    cuuint32_t estride[2] = {1, 1};
    CUresult r = get_encode()(&s->tmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, s->xb, gdim, gstride, box, estride,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
    e = cudaFuncSetAttribute(tc::logreg_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    s->ok = true;
  }
  int blocks = (points + tc::BN - 1) / tc::BN;
  if (blocks * tc::BN > s->bsplit_pts) {
    cudaFree(s->bsplit);
    s->bsplit = nullptr;
    e = cudaMalloc(&s->bsplit, sizeof(__nv_bfloat16) * (size_t)blocks * tc::BN * tc::NSPLIT * tc::BK);
    if (e != cudaSuccess) return e;
    cudaMemset(s->bsplit, 0, sizeof(__nv_bfloat16) * (size_t)blocks * tc::BN * tc::NSPLIT * tc::BK);
    s->bsplit_pts = blocks * tc::BN;
  }
  return e;
}

void logreg_tc_free(ModelDev& m) {
  tc::TCState* s = reinterpret_cast<tc::TCState*>(m.tc);
  if (!s) return;
  cudaFree(s->xb);
  cudaFree(s->lin);
  cudaFree(s->bsplit);
  cudaFree(s->err);
  delete s;
  m.tc = nullptr;
}

int logreg_tc_error(const ModelDev& m) {
  tc::TCState* s = reinterpret_cast<tc::TCState*>(m.tc);
  if (!s) return 0;
  int v = 0;
  cudaMemcpy(&v, s->err, sizeof(int), cudaMemcpyDeviceToHost);
  return v;
}

void logreg_finish_launch(const float* Q, int npts, int ld, int p, int row_groups, const float* part_g,
                          const double* part_ll, const double* lin, double prior_scale, double* PE, float* G,
                          const int32_t* pending, cudaStream_t st);

cudaError_t logreg_tc_launch(ModelDev& m, const float* Q, int npts, double* PE, float* G, const int32_t* pending,
                             cudaStream_t st) {
  tc::TCState* s = reinterpret_cast<tc::TCState*>(m.tc);
  if (!s || !s->ok) return cudaErrorNotSupported;
  cudaError_t e = logreg_tc_prepare(m, npts);
  if (e != cudaSuccess) return e;
  int blocks = (npts + tc::BN - 1) / tc::BN;
  int64_t ntiles = (m.n + tc::BM - 1) / tc::BM;
  int rg = std::max(1, 152 / blocks);
  if (rg > ntiles) rg = (int)ntiles;
  if (rg > m.row_groups) rg = m.row_groups;  // partial buffers are sized for m.row_groups
  int npad = blocks * tc::BN;
  tc::split_coefs_kernel<<<(npad * tc::BK + 255) / 256, 256, 0, st>>>(Q, npts, m.D, m.p, npad, s->bsplit, pending);
  tc::Params P{m.n, s->bsplit, npts, rg, m.part_g, m.part_ll, s->err, pending};
  tc::logreg_tc_kernel<<<dim3(blocks, rg), tc::NUM_THREADS, tc::SMEM_BYTES, st>>>(s->tmap, P);
  logreg_finish_launch(Q, npts, m.D, m.p, rg, m.part_g, m.part_ll, s->lin, m.hyper[0], PE, G, pending, st);
  return cudaGetLastError();
}

}  // namespace gbn
