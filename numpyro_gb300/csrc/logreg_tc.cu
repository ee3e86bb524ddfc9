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
//   warp 0      TMA producer: X' tile [128 rows x 64 feat] bf16, 128B swizzle, 8-stage ring,
//               with an L2 prefetch running 8 tiles ahead
//   warp 1      MMA issuer:  GEMM1  H[128 chains x 128 rows] = (b_hi + b_mid + b_lo)/2 . X'_tile^T
//                            (three K=64 BF16 products accumulate in FP32 in TMEM, so the
//                            FP32 coefficients are represented exactly: "bf16x3"),
//                            GEMM2  G[128 chains x 64 feat] += E . X'_tile  (E = sigmoid(l'),
//                            the A operand read from TMEM)
//   warps 2..17 epilogue: TMEM lanes are chains, columns rows.  Two groups of 8 warps take
//               alternate tiles; in a group 2 warps per lane quadrant split the 128 rows.  Per
//               logit one ex2 and one tanh; log(1 + e^{-|l'|}) is taken as one lg2 of the product
//               of 8 rows' factors (2.125 special-function ops per logit).  E goes back to TMEM
//               as bf16 pairs, into columns of the same H buffer the warp has already read.
//               Each thread accumulates its chain's log-likelihood over its rows; the four
//               threads of a chain are combined once per CTA in FP64.
// Three H buffers in TMEM (3 x 128 columns) keep three tiles in flight, and GEMM2 of tile t is
// issued after GEMM1 of tile t + 2; G lives in TMEM for the whole launch (64 columns).  Keeping
// E in TMEM leaves shared memory to the X' and coefficient operands: with E in shared memory
// as well (its stores plus GEMM2 reading it), the tensor pipe waited on shared-memory bandwidth.
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
constexpr int EPI_GROUP = EPI_WARPS / 2;  // warps that share one tile (groups take alternate tiles)
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
static_assert(NUM_BARS * 8 + 8 <= 256, "barriers, TMEM address and abort flag fit their slot");

// One part of the epilogue for one warp: its lane's chain x 32 rows (TMEM columns at th).
// TMEM holds h = l'/2 (the coefficients enter GEMM1 halved, an exact scaling).  Per row:
//   E = sigmoid(l') = tanh(h)/2 + 1/2                      -> bf16, GEMM2's A operand in TMEM
//       (forming it from e^{-2|h|} on the FMA pipe, with one reciprocal per 8 rows or by
//       Newton's method, measured slower)
//   softplus(l') - l'/2 = |h| + log(1 + e^{-2|h|})          -> |h| summed, the logs taken as
//                                                            one log2 per product of 8 rows
// With MASK, rows r >= nvalid lie past the end of the data: they are left out of the
// log-likelihood (their X' rows are zero, so E needs no mask).
// E goes to the 16 TMEM columns at te, two rows per column (the even row in the low half):
// columns this warp has already read, so H and E share the buffer.
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
#pragma unroll
  for (int g8 = 0; g8 < 4; ++g8) {
    float prod = 1.0f;
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
      pk[4 * g8 + (e >> 1)] = pack_bf16(ev[0], ev[1]);
    }
    tl += lg2_approx(prod);
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
          // A = E rows 16kk..16kk+15: 8 TMEM columns in row half kk / 4 (rows 64 h + r at column
          // 64 h + r / 2); B = X' tile, MN-major (features contiguous), 8-row groups 1024 B apart
          mma_bf16_tmem_a_warp(tmem + ACC2_COL, ea + (uint32_t)((kk >> 2) * 64 + (kk & 3) * 8),
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
    // Two groups of 8 warps take alternate tiles, so that the groups' TMEM loads and
    // special-function bursts interleave instead of coinciding.
    // In a group, 2 warps per TMEM lane quadrant each take a 64-row half of the tile, as two
    // 32-row parts.
    const int ew = warp - 2;
    const int q = warp & 3;          // TMEM lane quadrant this warp may access: chains 32q..32q+31
    const int grp = ew / EPI_GROUP;  // tiles i with i % 2 == grp
    const int rh = (ew >> 2) & 1;    // row half of each tile: rows 64 rh .. 64 rh + 63
    const int c = q * 32 + lane;     // this thread's chain within the CTA
    const uint32_t tl = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(rh * 64);
    Comp32 ll{0.0f, 0.0f};  // log-likelihood of this chain over this thread's rows, all tiles
    bool ok = true;
    for (int i = grp; i < my_tiles && ok; i += 2) {
      const int64_t row0 = ((int64_t)rg + (int64_t)i * P.row_groups) * BM + rh * 64;
      const int b = i % NBUF;
      ok = bar_wait(bar(B_ACCF + b), (i / NBUF) & 1, abort_flag, P.err);
      if (!ok) break;
      tc_fence_after();
#pragma unroll
      for (int part = 0; part < 2; ++part) {
        float sabs = 0.0f, slg = 0.0f;
        const int64_t nleft = P.n - (row0 + part * 32);
        // H of rows 64 rh + 32 part .. +31 is read from columns 64 rh + 32 part; their E goes to
        // columns 64 rh + 16 part .. +15, which part 0 has already read
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

int* logreg_tc_error_ptr(const ModelDev& m) {
  tc::TCState* s = reinterpret_cast<tc::TCState*>(m.tc);
  return s ? s->err : nullptr;
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
  tc::Params P{m.n, s->bsplit, npts, rg, m.part_g, m.part_ll, s->err, pending};
  tc::logreg_tc_kernel<<<dim3(blocks, rg), tc::NUM_THREADS, tc::SMEM_BYTES, st>>>(s->tmap, P);
  if (!fused_tick)
    logreg_finish_launch(Q, npts, m.D, m.p, rg, m.part_g, m.part_ll, s->lin, m.hyper[0], PE, G, pending, st);
  return cudaGetLastError();
}

}  // namespace gbn
