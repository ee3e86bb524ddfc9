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
//   sum_n (sigmoid(l_n) - y_n) X_n = sum_n sigmoid(l'_n) X'_n = (sum_n tanh(l'_n/2) X'_n + X'^T 1) / 2
// so the kernel never reads y: it streams X', and the linear part sum_n l'_n / 2 = (X'^T 1 / 2) . b
// is added per chain from a vector computed once (lr_finish.cuh).
//
// One CTA owns 128 chains and a strided set of 128-row tiles of X':
//   warp 0      TMA producer: X' tile [128 rows x 64 feat] bf16, 128B swizzle, 8-stage ring,
//               with an L2 prefetch running 8 tiles ahead
//   warp 1      MMA issuer:  GEMM1  H[128 chains x 128 rows] = (b_hi + b_mid [+ b_lo])/2 . X'_tile^T
//                            (K = 64 BF16 products accumulating in FP32 in TMEM: with all three
//                            terms the FP32 coefficients are represented exactly; see below),
//                            GEMM2  G[128 chains x 64 feat] += E . X'_tile  (E = tanh(l'/2),
//                            the A operand read from TMEM)
//   warps 2..17 epilogue: TMEM lanes are chains, columns rows.  Two groups of 8 warps take
//               alternate tiles; in a group 2 warps per lane quadrant split the 128 rows.  Per
//               logit one ex2; E by tanh for half the rows and from the ex2 with one reciprocal
//               per 8 rows for the other half; log(1 + e^{-|l'|}) as one lg2 of the product of 8
//               rows' factors (1.6875 special-function ops per logit; epilogue_part).  E goes back
//               to TMEM as bf16 pairs, into columns of the same H buffer the warp has already read.
//               Each thread accumulates its chain's log-likelihood over its rows; the four
//               threads of a chain are combined once per CTA in FP64.
// Three H buffers in TMEM (3 x 128 columns) keep three tiles in flight, and GEMM2 of tile t is
// issued after GEMM1 of tile t + 2; G lives in TMEM for the whole launch (64 columns).  Keeping
// E in TMEM leaves shared memory to the X' and coefficient operands: with E in shared memory
// as well (its stores plus GEMM2 reading it), the tensor pipe waited on shared-memory bandwidth.
//
// Two or three coefficient terms.  b/2 = hi + mid + lo exactly (bf16 each, |lo| <= 2^-17 |b/2|).
// The third GEMM1 product (a third of GEMM1) is left out when the first-order term the finish adds
// in its place, nu(b_hm) . b_lo (lr_finish.cuh), is exact to 1e-3: the remainder of that expansion
// is at most (1/8) lambda_max(X^T X) |b_lo|^2 = (1/2) lambda_max |lo|^2, and the launch compares the
// largest |lo|^2 over a block's 128 chains with 2e-3 / lambda_hat, lambda_hat a Gershgorin bound on
// lambda_max(X^T X) formed once per model (far below the FP32 rounding of U's row sums).  The
// block's choice is recorded per launch (split3) for the finish.
// The design matrix must be exactly representable in bf16 (checked on the host).
// Every mbarrier wait is bounded; on a timeout the CTA records an error, drains its
// in-flight copies and MMAs (bounded), frees TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
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
constexpr int STAGES = 8;  // X' tiles stay resident until GEMM2, LAG tiles after GEMM1
constexpr int X_TILE = BM * BK * 2;  // 16 KB
constexpr int B_TILE = BN * BK * 2;  // 16 KB
constexpr int NBUF = 3;              // H buffers in TMEM (each also holds its tile's E): tiles in flight
constexpr int PREFETCH = 8;          // X' tiles an L2 prefetch runs ahead of the loads
constexpr int LAG = 2;               // GEMM2 of tile i - LAG is issued after GEMM1 of tile i
constexpr int OFF_X = 0;
constexpr int OFF_B = OFF_X + STAGES * X_TILE;
constexpr int OFF_MISC = OFF_B + NSPLIT * B_TILE;
constexpr int NUM_BARS = 2 * STAGES + 3 * NBUF + 1;
constexpr int SMEM_BYTES = OFF_MISC + 256 + BN * 8 + 1024;  // + alignment slack
constexpr int EPI_WARPS = 16;             // epilogue warps: 4 per TMEM lane quadrant
// EPI_ALTERNATE: two groups of 8 warps take alternate tiles (each warp 64 rows of every other
// tile); otherwise all 16 warps take every tile (each warp 32 rows of it).  Measured at 1024 chains
// x 581,012 rows: alternate 0.211 ms, every tile 0.226 ms (the groups' TMEM loads and
// special-function bursts interleave instead of coinciding).
constexpr bool EPI_ALTERNATE = true;
constexpr int EPI_GROUP = EPI_ALTERNATE ? EPI_WARPS / 2 : EPI_WARPS;  // warps that share one tile
constexpr int EPI_ROWS = BM * 4 / EPI_GROUP;                         // rows of a tile per warp
constexpr int GCOLS = BK * 4 / EPI_WARPS; // gradient columns read back per epilogue warp
constexpr int NUM_THREADS = 32 * (2 + EPI_WARPS);
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t ACC2_COL = NBUF * BM;  // G after the H buffers

// ACCF: GEMM1 wrote H; SF: the epilogue wrote E (into the same buffer); SE: GEMM2 has read E, the
// buffer is free for GEMM1 again
enum { B_XFULL = 0, B_XEMPTY = STAGES, B_ACCF = 2 * STAGES, B_SF = B_ACCF + NBUF, B_SE = B_SF + NBUF,
       B_DONE = B_SE + NBUF };
static_assert(LAG < NBUF, "GEMM1 of tile i reuses the buffer GEMM2 of tile i - NBUF reads");
static_assert(ACC2_COL + BK <= TMEM_COLS, "TMEM holds the H buffers and G");
static_assert(SMEM_BYTES <= 232448, "shared memory per CTA");
static_assert(NUM_BARS * 8 + 8 + 16 <= 256, "barriers, TMEM address, abort flag and |lo|^2 maxima fit their slot");

// One part of the epilogue for one warp: its lane's chain x 32 rows (TMEM columns at th).
// TMEM holds h = l'/2 (the coefficients enter GEMM1 halved, an exact scaling).  Per row:
//   softplus(l') - l'/2 = |h| + log(1 + t),  t = e^{-2|h|} = e^{-|l'|}   (one ex2)
//       |h| summed; the logs taken as one lg2 per product of 8 rows' (1 + t)
//   E = tanh(h) = 2 sigmoid(l') - 1   -> bf16, GEMM2's A operand in TMEM
//       (GEMM2 then gives sum_r tanh(h_r) X'_r = 2 (sum_r sigmoid(l'_r) X'_r) - X'^T 1: the
//        finish halves it and adds X'^T 1 / 2, the vector the linear term already uses)
// The 32 rows are 4 groups of 8.  tanh runs on the special-function unit at half the rate of
// ex2, so the first RCP_GROUPS groups form E from the t already computed instead: with
// u_j = 1 + t_j, one reciprocal R = 1 / (u_0 ... u_7) and prefix products P_j = u_0 ... u_j,
// 1 / u_j = P_{j-1} (R u_7 ... u_{j+1}) and tanh(|h_j|) = 2 / u_j - 1 (relative error ~1e-6,
// FP32 products).  The other groups use tanh.  With every group on one path or the other, one
// unit or the other was the wall (measured at 1024 chains x 581,012 rows: all tanh 0.253 ms, all
// reciprocal 0.282 ms; with the FP32 pair arithmetic below and two coefficient terms, one group
// in four 0.219 ms, two 0.213 ms).  Pairs of rows share FP32x2 instructions (ex2 arguments, the
// products) to save issue slots.
// With MASK, rows r >= nvalid lie past the end of the data: they are left out of the
// log-likelihood (their X' rows are zero, so E needs no mask).
// E goes to the 16 TMEM columns at te, two rows per column (the even row in the low half):
// columns this warp has already read, so H and E share the buffer.
constexpr int RCP_GROUPS = 2;

template <bool MASK>
__device__ __forceinline__ void epilogue_part(uint32_t th, uint32_t te, int nvalid, float& sabs, float& slg) {
  const float NEG_2LOG2E = -2.8853900817779268f;
  uint32_t v[2][16];
  tmem_ld16u(th, v[0]);
  tmem_ld16u(th + 16, v[1]);
  tmem_wait16(v[0]);
  tmem_wait16(v[1]);
  float ta = 0.0f, tl = 0.0f;
  uint32_t pk[16];
  int g_first = 0;  // the first group the loop below takes
  if (RCP_GROUPS == 2 && (!MASK || nvalid >= 16)) {
    // groups 0 and 1 in the reciprocal form side by side, in the two halves of FP32x2 instructions
    const float2 C2 = make_float2(NEG_2LOG2E, NEG_2LOG2E);
    float ha[8], hb[8];
    float2 tv[8], pp[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      ha[j] = __uint_as_float(v[0][j]);
      hb[j] = __uint_as_float(v[0][8 + j]);
      const float2 a = __fmul2_rn(make_float2(ha[j], hb[j]), C2);
      tv[j] = make_float2(ex2_approx(-fabsf(a.x)), ex2_approx(-fabsf(a.y)));
      ta += fabsf(ha[j]);
      ta += fabsf(hb[j]);
    }
    pp[0] = __fadd2_rn(make_float2(1.0f, 1.0f), tv[0]);
#pragma unroll
    for (int j = 1; j < 8; ++j) pp[j] = __ffma2_rn(pp[j - 1], tv[j], pp[j - 1]);
    float2 q = make_float2(rcp_approx(pp[7].x), rcp_approx(pp[7].y));  // 1 / P_j, from j = 7 down
    float ea[8], eb[8];
#pragma unroll
    for (int j = 7; j >= 0; --j) {
      const float2 inv_u = j == 0 ? q : __fmul2_rn(pp[j > 0 ? j - 1 : 0], q);
      const float2 e = __ffma2_rn(inv_u, make_float2(2.0f, 2.0f), make_float2(-1.0f, -1.0f));
      ea[j] = copysignf(e.x, ha[j]);
      eb[j] = copysignf(e.y, hb[j]);
      if (j > 0) q = __ffma2_rn(q, tv[j], q);
    }
#pragma unroll
    for (int j = 0; j < 8; j += 2) {
      pk[j >> 1] = pack_bf16(ea[j], ea[j + 1]);
      pk[4 + (j >> 1)] = pack_bf16(eb[j], eb[j + 1]);
    }
    tl += lg2_approx(pp[7].x * pp[7].y);
    g_first = 2;
  }
#pragma unroll
  for (int g8 = 0; g8 < 4; ++g8) {
    if (g8 < g_first) continue;
    const bool full = !MASK || 8 * g8 + 8 <= nvalid;
    if (g8 < RCP_GROUPS && full) {
      float hv[8], tv[8], pp[8];
#pragma unroll
      for (int j = 0; j < 8; j += 2) {
        const int r = 8 * g8 + j;
        hv[j] = __uint_as_float(v[r >> 4][r & 15]);
        hv[j + 1] = __uint_as_float(v[(r + 1) >> 4][(r + 1) & 15]);
        const float2 a = __fmul2_rn(make_float2(hv[j], hv[j + 1]), make_float2(NEG_2LOG2E, NEG_2LOG2E));
        tv[j] = ex2_approx(-fabsf(a.x));
        tv[j + 1] = ex2_approx(-fabsf(a.y));
        ta += fabsf(hv[j]);
        ta += fabsf(hv[j + 1]);
      }
      pp[0] = 1.0f + tv[0];
#pragma unroll
      for (int j = 1; j < 8; ++j) pp[j] = fmaf(pp[j - 1], tv[j], pp[j - 1]);
      float q = rcp_approx(pp[7]);  // q = 1 / P_j, from j = 7 down
      float ev[8];
#pragma unroll
      for (int j = 7; j >= 0; --j) {
        const float inv_u = j == 0 ? q : pp[j > 0 ? j - 1 : 0] * q;
        ev[j] = copysignf(fmaf(2.0f, inv_u, -1.0f), hv[j]);
        if (j > 0) q = fmaf(q, tv[j], q);
      }
#pragma unroll
      for (int j = 0; j < 8; j += 2) pk[4 * g8 + (j >> 1)] = pack_bf16(ev[j], ev[j + 1]);
      tl += lg2_approx(pp[7]);
    } else if (full) {
      float2 prod = make_float2(1.0f, 1.0f);
#pragma unroll
      for (int e = 0; e < 8; e += 2) {
        const int r = 8 * g8 + e;
        const float h0 = __uint_as_float(v[r >> 4][r & 15]), h1 = __uint_as_float(v[(r + 1) >> 4][(r + 1) & 15]);
        const float2 a = __fmul2_rn(make_float2(h0, h1), make_float2(NEG_2LOG2E, NEG_2LOG2E));
        const float t0 = ex2_approx(-fabsf(a.x)), t1 = ex2_approx(-fabsf(a.y));  // e^{-|l'|}
        ta += fabsf(h0);
        ta += fabsf(h1);
        prod = __ffma2_rn(prod, make_float2(t0, t1), prod);  // prod * (1 + t), one rounding
        pk[4 * g8 + (e >> 1)] = pack_bf16(tanh_approx(h0), tanh_approx(h1));
      }
      tl += lg2_approx(prod.x * prod.y);
    } else {
      float prod = 1.0f;
#pragma unroll
      for (int e = 0; e < 8; e += 2) {
        float ev[2];
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
          const int r = 8 * g8 + e + hh;
          const float h = __uint_as_float(v[r >> 4][r & 15]);
          if (r < nvalid) {
            ta += fabsf(h);
            prod = fmaf(prod, ex2_approx(fabsf(h) * NEG_2LOG2E), prod);
          }
          ev[hh] = tanh_approx(h);
        }
        pk[4 * g8 + (e >> 1)] = pack_bf16(ev[0], ev[1]);
      }
      tl += lg2_approx(prod);
    }
  }
  tmem_st16(te, pk);
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
  float lo2_limit;  // largest |lo|^2 of a block's chains for two coefficient terms (< 0: always three)
  int32_t* split3;  // [chain blocks]: 1 where the launch took three terms (written by row group 0)
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
    for (int i = 0; i < NBUF; ++i) {
      bar_init(bar(B_ACCF + i), 1);
      bar_init(bar(B_SF + i), EPI_GROUP);
      bar_init(bar(B_SE + i), 1);
    }
    bar_init(bar(B_DONE), 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  float* lo2_slot = reinterpret_cast<float*>(smem + OFF_MISC + NUM_BARS * 8 + 8);
  for (int i = threadIdx.x; i < BN; i += NUM_THREADS) ll_smem[i] = 0.0;
  // |lo|^2 of each chain of the block (threads 0..127, four whole warps), maximum per warp
  if (threadIdx.x < BN) {
    const uint4* lo = reinterpret_cast<const uint4*>(P.bsplit + ((size_t)(cb * BN + threadIdx.x) * NSPLIT + 2) * BK);
    float s2 = 0.0f;
#pragma unroll
    for (int k = 0; k < BK / 8; ++k) {
      const uint4 u = lo[k];
      const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float a = __uint_as_float(w[j] << 16), b = __uint_as_float(w[j] & 0xffff0000u);
        s2 = fmaf(a, a, fmaf(b, b, s2));
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s2 = fmaxf(s2, __shfl_xor_sync(0xffffffffu, s2, o));
    if (lane == 0) lo2_slot[warp] = s2;
  }
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
  const float lo2max = fmaxf(fmaxf(lo2_slot[0], lo2_slot[1]), fmaxf(lo2_slot[2], lo2_slot[3]));
  const int nsplit = lo2max > P.lo2_limit ? 3 : 2;
  if (threadIdx.x == 0 && rg == 0 && P.split3) P.split3[cb] = nsplit == 3 ? 1 : 0;

  if (warp == 0) {
    // ------------------------------------------------------------ TMA producer
    if (lane == 0) {
      int issued = 0;
      for (int i = 0; i < my_tiles; ++i) {
        int s = i % STAGES;
        if (i >= STAGES && !bar_wait(bar(B_XEMPTY + s), ((i / STAGES) - 1) & 1, abort_flag, P.err)) break;
        int64_t row0 = ((int64_t)rg + (int64_t)i * P.row_groups) * BM;
        // X' tiles are held until GEMM2, so a stage frees only a little ahead of its next use:
        // pull the tile PREFETCH loads ahead into L2 now, so the load later hits L2
        if (i + PREFETCH < my_tiles)
          tma_prefetch_2d(&tmap_x, 0, (int)(row0 + (int64_t)PREFETCH * P.row_groups * BM));
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
    constexpr uint32_t ID2 = idesc(BN, BK, 0, 1);  // G = E . X': E K-major in TMEM, X' MN-major
    const uint32_t xb = smem_u32(smem + OFF_X), bb = smem_u32(smem + OFF_B);
    const uint64_t dcoef = sdesc(bb, 16, 1024);  // GEMM1 A: the coefficient splits, the same every tile
    const uint64_t dx1 = sdesc(xb, 16, 1024);    // GEMM1 B: X' tile, K-major, stage 0
    const uint64_t dx2 = sdesc(xb, 1024, 1024);  // GEMM2 B: X' tile, MN-major, stage 0
    bool ok = true;
    // Tile i uses H buffer i % NBUF; the k-th use of a buffer completes its barriers' phase k.
    // GEMM2 takes its A operand (E) from TMEM, where the epilogue wrote it into the tile's own H
    // buffer, so shared memory carries only the X' and coefficient operands (as operands, both
    // GEMMs read shared memory at close to its bandwidth).  GEMM1(i) first waits for X' tile i
    // and for GEMM2 of tile i - NBUF to have read the buffer; GEMM2(i - LAG) then waits for its
    // E.  The chain epilogue -> GEMM2 -> GEMM1 -> epilogue so spans LAG + 1 tiles.  tcgen05.mma
    // issue is paced by execution (a shallow queue); stages, buffers and parities are counters.
    int si = 0, pi = 0, bi = 0, qi = 0;  // tile i: X' stage, its fill parity; H buffer, its use parity
    int sj = 0, bj = 0, qj = 0;          // tile j = i - LAG: X' stage; buffer, its use parity
    for (int i = 0; i < my_tiles + LAG; ++i) {
      if (i < my_tiles) {
        ok = bar_wait3_warp(bar(B_XFULL + si), pi, true, bar(B_SE + bi), qi ^ 1, i >= NBUF, 0u, 0u, false,
                            abort_flag, P.err);
        if (!ok) break;
        tc_fence_after();
        const uint32_t d = tmem + (uint32_t)(bi * BM);
        const uint64_t xs = sdesc_at(dx1, (uint32_t)(si * X_TILE));
#pragma unroll
        for (int k = 0; k < NSPLIT; ++k) {
          if (k >= nsplit) break;
#pragma unroll
          for (int kk = 0; kk < BK / 16; ++kk)
            mma_bf16_warp(d, sdesc_at(dcoef, k * B_TILE + kk * 32), sdesc_at(xs, kk * 32), ID1,
                          (k | kk) ? 1u : 0u);
        }
        mma_commit_warp(bar(B_ACCF + bi));
        if (++si == STAGES) si = 0, pi ^= 1;
        if (++bi == NBUF) bi = 0, qi ^= 1;
      }
      if (i >= LAG) {
        const int j = i - LAG;
        ok = bar_wait_warp(bar(B_SF + bj), qj, abort_flag, P.err);  // E of tile j is in TMEM
        if (!ok) break;
        tc_fence_after();
        const uint32_t ea = tmem + (uint32_t)(bj * BM);
        const uint64_t xs = sdesc_at(dx2, (uint32_t)(sj * X_TILE));
#pragma unroll
        for (int kk = 0; kk < BM / 16; ++kk) {
          // A = E rows 16kk..16kk+15: 8 TMEM columns in the block of the warp that wrote them
          // (rows EPI_ROWS w + r at column EPI_ROWS w + r / 2); B = X' tile, MN-major (features
          // contiguous), 8-row groups 1024 B apart
          constexpr int KW = EPI_ROWS / 16;  // K steps per epilogue warp's block of rows
          mma_bf16_tmem_a_warp(tmem + ACC2_COL, ea + (uint32_t)((kk / KW) * EPI_ROWS + (kk % KW) * 8),
                               sdesc_at(xs, kk * 2048), ID2, (j > 0 || kk > 0) ? 1u : 0u);
        }
        mma_commit_warp(bar(B_SE + bj));
        mma_commit_warp(bar(B_XEMPTY + sj));
        if (++sj == STAGES) sj = 0;
        if (++bj == NBUF) bj = 0, qj ^= 1;
      }
    }
    __syncwarp();
    mma_commit_warp(bar(B_DONE));
    // wait for every MMA issued by this warp before TMEM can be released
    for (uint32_t k = 0; k < WAIT_LIMIT && !bar_try(bar(B_DONE), 0); ++k) {
    }
  } else {
    // ------------------------------------------------------------ epilogue (warps 2..17)
    // The EPI_GROUP warps that take a tile split its rows: EPI_ROWS per warp, the warps of each
    // TMEM lane quadrant side by side, as 32-row parts.
    const int ew = warp - 2;
    const int q = warp & 3;                                  // TMEM lane quadrant: chains 32q..32q+31
    const int grp = EPI_ALTERNATE ? ew / EPI_GROUP : 0;      // tiles i with i % NGRP == grp
    constexpr int NGRP = EPI_WARPS / EPI_GROUP;
    const int wr = (ew >> 2) % (EPI_GROUP / 4);              // this warp's block of rows in a tile
    const int c = q * 32 + lane;                             // this thread's chain within the CTA
    const uint32_t tl = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(wr * EPI_ROWS);
    Comp32 ll{0.0f, 0.0f};  // log-likelihood of this chain over this thread's rows, all tiles
    bool ok = true;
    for (int i = grp; i < my_tiles && ok; i += NGRP) {
      const int64_t row0 = ((int64_t)rg + (int64_t)i * P.row_groups) * BM + wr * EPI_ROWS;
      const int b = i % NBUF;
      ok = bar_wait(bar(B_ACCF + b), (i / NBUF) & 1, abort_flag, P.err);
      if (!ok) break;
      tc_fence_after();
#pragma unroll
      for (int part = 0; part < EPI_ROWS / 32; ++part) {
        float sabs = 0.0f, slg = 0.0f;
        const int64_t nleft = P.n - (row0 + part * 32);
        // H of the block's rows 32 part .. +31 is read from its columns 32 part ..; their E goes
        // to its columns 16 part .. +15, which this warp has already read
        const uint32_t th = tl + (uint32_t)(b * BM + part * 32), te = tl + (uint32_t)(b * BM + part * 16);
        if (nleft >= 32)
          epilogue_part<false>(th, te, 32, sabs, slg);
        else
          epilogue_part<true>(th, te, nleft > 0 ? (int)nleft : 0, sabs, slg);
        ll.add(fmaf(0.6931471805599453f, slg, sabs));
      }
      tmem_wait_st();  // E is in TMEM before GEMM2 may read it
      tc_fence_before();
      __syncwarp();
      if (lane == 0) bar_arrive(bar(B_SF + b));
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

// X^T X (p <= 64) in FP64 from FP32 partials over 32-row chunks staged in shared memory, for the
// Gershgorin bound on its largest eigenvalue.  256 threads, 16 entries of the 64 x 64 matrix each.
__global__ void __launch_bounds__(256) gram_kernel(const float* __restrict__ x, int64_t n, int p,
                                                   double* __restrict__ gram) {
  __shared__ float xs[32][BK];
  float acc[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) acc[k] = 0.0f;
  for (int64_t r0 = (int64_t)blockIdx.x * 32; r0 < n; r0 += (int64_t)gridDim.x * 32) {
    __syncthreads();
    for (int i = threadIdx.x; i < 32 * BK; i += blockDim.x) {
      const int rr = i / BK, d = i % BK;
      const int64_t r = r0 + rr;
      xs[rr][d] = (r < n && d < p) ? x[r * p + d] : 0.0f;
    }
    __syncthreads();
    for (int rr = 0; rr < 32; ++rr) {
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        const int e = threadIdx.x + k * 256;
        acc[k] = fmaf(xs[rr][e / BK], xs[rr][e % BK], acc[k]);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    const int e = threadIdx.x + k * 256;
    if (e / BK < p && e % BK < p) atomicAdd(&gram[e], (double)acc[k]);
  }
}

struct TCState {
  double* lin = nullptr;
  __nv_bfloat16* xb = nullptr;
  __nv_bfloat16* bsplit = nullptr;
  int32_t* split3 = nullptr;  // [bsplit_pts / 128]
  float lo2_limit = -1.0f;    // < 0: always three coefficient terms
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
    // two coefficient terms where |lo|^2 <= 2 tau / lambda_hat, tau = 1e-3 (see the file header);
    // GBN_LOGREG_TERMS=3 keeps all three
    const char* terms = getenv("GBN_LOGREG_TERMS");
    if (!(terms && terms[0] == '3')) {
      double* gram = nullptr;
      e = cudaMalloc(&gram, sizeof(double) * tc::BK * tc::BK);
      if (e != cudaSuccess) return e;
      cudaMemset(gram, 0, sizeof(double) * tc::BK * tc::BK);
      tc::gram_kernel<<<304, 256>>>(m.x, m.n, m.p, gram);
      std::vector<double> g((size_t)tc::BK * tc::BK);
      e = cudaMemcpy(g.data(), gram, sizeof(double) * g.size(), cudaMemcpyDeviceToHost);
      cudaFree(gram);
      if (e != cudaSuccess) return e;
      double lam = 0.0;  // Gershgorin: lambda_max <= max_i sum_j |G_ij|
      for (int i = 0; i < m.p; ++i) {
        double row = 0.0;
        for (int j = 0; j < m.p; ++j) row += std::fabs(g[(size_t)i * tc::BK + j]);
        lam = std::max(lam, row);
      }
      lam *= 1.01;  // the FP32 partial sums' rounding
      s->lo2_limit = lam > 0.0 ? (float)(2.0e-3 / lam) : 3.0e38f;
    }
    s->ok = true;
  }
  int blocks = (points + tc::BN - 1) / tc::BN;
  if (blocks * tc::BN > s->bsplit_pts) {
    cudaFree(s->bsplit);
    s->bsplit = nullptr;
    e = cudaMalloc(&s->bsplit, sizeof(__nv_bfloat16) * (size_t)blocks * tc::BN * tc::NSPLIT * tc::BK);
    if (e != cudaSuccess) return e;
    cudaMemset(s->bsplit, 0, sizeof(__nv_bfloat16) * (size_t)blocks * tc::BN * tc::NSPLIT * tc::BK);
    cudaFree(s->split3);
    s->split3 = nullptr;
    e = cudaMalloc(&s->split3, sizeof(int32_t) * (size_t)blocks);
    if (e != cudaSuccess) return e;
    cudaMemset(s->split3, 0, sizeof(int32_t) * (size_t)blocks);
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
  cudaFree(s->split3);
  cudaFree(s->err);
  delete s;
  m.tc = nullptr;
}

int* logreg_tc_error_ptr(const ModelDev& m) {
  tc::TCState* s = reinterpret_cast<tc::TCState*>(m.tc);
  return s ? s->err : nullptr;
}

cudaError_t logreg_tc_terms(const ModelDev& m, int* three, int* blocks, float* limit) {
  tc::TCState* s = reinterpret_cast<tc::TCState*>(m.tc);
  *three = 0;
  *blocks = 0;
  *limit = s ? s->lo2_limit : -1.0f;
  if (!s || !s->split3) return cudaSuccess;
  std::vector<int32_t> v((size_t)s->bsplit_pts / tc::BN);
  cudaError_t e = cudaMemcpy(v.data(), s->split3, sizeof(int32_t) * v.size(), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return e;
  for (int32_t x : v) *three += x != 0;
  *blocks = (int)v.size();
  return cudaSuccess;
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
                          const int32_t* pending, cudaStream_t st, const int32_t* split3, bool e_tanh);

// row groups of a launch over npts points: the grid fills the SMs with (chain blocks x row groups)
static int logreg_tc_row_groups(const ModelDev& m, int npts) {
  const int blocks = (npts + tc::BN - 1) / tc::BN;
  const int64_t ntiles = (m.n + tc::BM - 1) / tc::BM;
  int rg = std::max(1, 152 / blocks);
  if (rg > ntiles) rg = (int)ntiles;
  if (rg > m.row_groups) rg = m.row_groups;  // partial buffers are sized for m.row_groups
  return rg;
}

void logreg_prior_consts(double prior_scale, int p, float* inv_var_f, double* pe_const);

bool logreg_tc_fusion(const ModelDev& m, int npts, AdvParams* P) {
  tc::TCState* s = reinterpret_cast<tc::TCState*>(m.tc);
  if (!s || !s->ok || !s->bsplit || !m.part_g) return false;
  P->lrf_part_g = m.part_g;
  P->lrf_part_ll = m.part_ll;
  P->lrf_lin = s->lin;
  P->lrf_bsplit = reinterpret_cast<uint16_t*>(s->bsplit);
  P->lrf_row_groups = logreg_tc_row_groups(m, npts);
  P->lrf_split3 = s->split3;
  P->lrf_e_tanh = 1;
  logreg_prior_consts(m.hyper[0], m.p, &P->lrf_inv_var, &P->lrf_pe_const);
  return true;
}

cudaError_t logreg_tc_launch(ModelDev& m, const float* Q, int npts, double* PE, float* G, const int32_t* pending,
                             cudaStream_t st, bool fused_tick) {
  tc::TCState* s = reinterpret_cast<tc::TCState*>(m.tc);
  if (!s || !s->ok) return cudaErrorNotSupported;
  cudaError_t e = logreg_tc_prepare(m, npts);
  if (e != cudaSuccess) return e;
  const int blocks = (npts + tc::BN - 1) / tc::BN;
  const int rg = logreg_tc_row_groups(m, npts);
  const int npad = blocks * tc::BN;
  // In the tick engine's fused form the state-machine kernel writes the coefficient splits with
  // the positions and finishes the sums, so only the tensor-core kernel runs here.
  if (!fused_tick)
    tc::split_coefs_kernel<<<(npad * tc::BK + 255) / 256, 256, 0, st>>>(Q, npts, m.D, m.p, npad, s->bsplit,
                                                                         pending);
  tc::Params P{m.n, s->bsplit, npts, rg, m.part_g, m.part_ll, s->err, pending, s->lo2_limit, s->split3};
  tc::logreg_tc_kernel<<<dim3(blocks, rg), tc::NUM_THREADS, tc::SMEM_BYTES, st>>>(s->tmap, P);
  if (!fused_tick)
    logreg_finish_launch(Q, npts, m.D, m.p, rg, m.part_g, m.part_ll, s->lin, m.hyper[0], PE, G, pending, st,
                         s->split3, true);
  return cudaGetLastError();
}

}  // namespace gbn
