// nuts_engine.cu -- the per-chain NUTS/HMC state machine ("advance" kernel).
//
// One group of threads (a warp, or a CTA for large D) owns one chain.  A
// launch of advance_kernel consumes the gradient the potential kernel just
// produced at the chain's query point, finishes that leapfrog step, runs the
// tree logic, and stops at the next point where the chain needs a gradient
// (its next leaf), writing that position into the query buffer Q.  The host
// alternates advance / potential launches ("ticks").
//
// In the fused engine each chain doubles its own tree and starts its next
// transition as soon as its tree ends, so every tick is a gradient for every
// live chain.  In the plain engine (lockstep=1) a chain that finished its
// transition waits until all chains have (numpyro's vmap'd while_loop
// semantics, numpyro/infer/hmc.py:796-798), and the potential is evaluated
// for every chain (masked lanes included).
//
// Reference arithmetic (numpyro/infer/hmc_util.py):
//   velocity_verlet.update_fn :289-309, _build_basetree :851-894,
//   _combine_tree :767-848 (uniform :749-753, biased :756-764),
//   _iterative_build_subtree :984-1085, _leaf_idx_to_ckpt_idxs :941-958,
//   _is_iterative_turning :961-981, _is_turning/_momentum_angle :710-746,
//   build_tree :1088-1180, euclidean_kinetic_energy :1183-1223,
//   dual_averaging :60-130, welford_covariance :133-239,
//   warmup_adapter.update_fn :637-705, find_reasonable_step_size :314-384;
// numpyro/infer/hmc.py: momentum_generator :92-110, _hmc_next :364-414,
//   _nuts_next :416-455, sample_kernel :459-530.
#include <cuda_bf16.h>

#include "common.cuh"
#include "hier_potential.cuh"
#include "internal.h"
#include "hs_finish.cuh"
#include "lr_finish.cuh"
#include "sv_potential.cuh"

namespace gbn {

constexpr float FLT32_TINY = 1.17549435e-38f;
constexpr float FLT32_MAX = 3.40282347e+38f;

// ------------------------------------------------------------------ dense mass matrix
// From a symmetric positive-definite covariance A (FP64, row-major [ld][ld], both triangles),
// writes the three HMCAdaptState matrices the way welford_covariance.final_fn and
// _initialize_mass_matrix do (numpyro/infer/hmc_util.py:199-239, :439-515):
//   inverse_mass_matrix  = A
//   mass_matrix_sqrt_inv = T, lower triangular with A = T^T T (the Cholesky factor of A with its
//                          index order reversed: A = U U^T, U upper, T = U^T)
//   mass_matrix_sqrt     = S = T^-1 (lower), so M = A^-1 = S S^T and momentum r = S eps.
// The factorisation runs in FP64 in place (U in the upper triangle, S below the diagonal); A is
// zeroed afterwards (it is the Welford m2 buffer, reset at every window end).  One group per
// matrix; threads own columns.
template <int NT>
__device__ void dense_factor(const Group<NT>& g, double* A, int D, int ld, float* inv, float* sq, float* sqi) {
  for (int j = g.tid; j < D; j += NT)
    for (int i = 0; i < D; ++i) inv[(size_t)i * ld + j] = (float)A[(size_t)i * ld + j];
  for (int k = D - 1; k >= 0; --k) {
    g.sync();
    const double ukk = sqrt(A[(size_t)k * ld + k]);
    for (int i = g.tid; i < k; i += NT) A[(size_t)i * ld + k] /= ukk;  // U[i][k]
    g.sync();
    if (g.tid == 0) A[(size_t)k * ld + k] = ukk;
    // trailing update of the leading k x k block (upper triangle): A[i][j] -= U[i][k] U[j][k]
    for (int j = g.tid; j < k; j += NT) {
      const double ujk = A[(size_t)j * ld + k];
      for (int i = 0; i <= j; ++i) A[(size_t)i * ld + j] -= A[(size_t)i * ld + k] * ujk;
    }
  }
  g.sync();
  // S = T^-1 column by column (T[r][m] = U[m][r] = A[m][r] for m <= r); S[r][c] -> A[r][c], r > c
  for (int cc = g.tid; cc < D; cc += NT) {
    const double scc = 1.0 / A[(size_t)cc * ld + cc];
    for (int r = cc + 1; r < D; ++r) {
      double acc = A[(size_t)cc * ld + r] * scc;  // m = cc
      for (int m = cc + 1; m < r; ++m) acc += A[(size_t)m * ld + r] * A[(size_t)m * ld + cc];
      A[(size_t)r * ld + cc] = -acc / A[(size_t)r * ld + r];
    }
    for (int r = 0; r < D; ++r) {
      const size_t o = (size_t)r * ld + cc;
      sqi[o] = (r >= cc) ? (float)A[(size_t)cc * ld + r] : 0.0f;
      sq[o] = (r > cc) ? (float)A[o] : (r == cc ? (float)scc : 0.0f);
    }
  }
  g.sync();
  for (int j = g.tid; j < D; j += NT)
    for (int i = 0; i < D; ++i) A[(size_t)i * ld + j] = 0.0;
  g.sync();
}

template <int NT, bool DM = false>  // DM: dense mass matrices
struct Chain {
  const AdvParams& P;
  Group<NT> g;
  double* red;
  int c;   // chain index
  int D;   // this chain's latent dim
  int ld;  // row stride of [C][ld] buffers
  ChainCtl ctl;
  // The twelve tree vectors (frontiers, proposals, momentum sums) are this chain's rows of the
  // EngineBufs [C][ld] buffers, or, when oc is set, consecutive rows of ld floats on chip.
  float* oc;
  __device__ __forceinline__ float* z_l_() const { return oc ? oc + 0 * (size_t)ld : V(P.e.z_l); }
  __device__ __forceinline__ float* r_l_() const { return oc ? oc + 1 * (size_t)ld : V(P.e.r_l); }
  __device__ __forceinline__ float* g_l_() const { return oc ? oc + 2 * (size_t)ld : V(P.e.g_l); }
  __device__ __forceinline__ float* z_r_() const { return oc ? oc + 3 * (size_t)ld : V(P.e.z_r); }
  __device__ __forceinline__ float* r_r_() const { return oc ? oc + 4 * (size_t)ld : V(P.e.r_r); }
  __device__ __forceinline__ float* g_r_() const { return oc ? oc + 5 * (size_t)ld : V(P.e.g_r); }
  __device__ __forceinline__ float* z_p_() const { return oc ? oc + 6 * (size_t)ld : V(P.e.z_p); }
  __device__ __forceinline__ float* g_p_() const { return oc ? oc + 7 * (size_t)ld : V(P.e.g_p); }
  __device__ __forceinline__ float* z_sp_() const { return oc ? oc + 8 * (size_t)ld : V(P.e.z_sp); }
  __device__ __forceinline__ float* g_sp_() const { return oc ? oc + 9 * (size_t)ld : V(P.e.g_sp); }
  __device__ __forceinline__ float* rsum_() const { return oc ? oc + 10 * (size_t)ld : V(P.e.rsum); }
  __device__ __forceinline__ float* rsum_sub_() const { return oc ? oc + 11 * (size_t)ld : V(P.e.rsum_sub); }
  __device__ __forceinline__ float* Q_() const { return V(P.e.Q); }
  __device__ __forceinline__ float* G_() const { return V(P.e.G); }

  __device__ __forceinline__ size_t row() const { return (size_t)c * ld; }

  // q[d] = v for the potential; when the tensor-core logistic potential is fused into the tick,
  // also the exact hi/mid/lo bfloat16 terms of v / 2 that its GEMM reads (as split_coefs_kernel)
  __device__ __forceinline__ void put_q(float* q, int d, float v) const {
    q[d] = v;
    if (P.lrf_bsplit) {
      const float h = 0.5f * v;
      const __nv_bfloat16 hi = __float2bfloat16_rn(h);
      const float r1 = h - __bfloat162float(hi);
      const __nv_bfloat16 mid = __float2bfloat16_rn(r1);
      const float r2 = r1 - __bfloat162float(mid);
      const __nv_bfloat16 lo = __float2bfloat16_rn(r2);
      uint16_t* o = P.lrf_bsplit + (size_t)c * 192 + d;
      o[0] = __bfloat16_as_ushort(hi);
      o[64] = __bfloat16_as_ushort(mid);
      o[128] = __bfloat16_as_ushort(lo);
    }
  }
  __device__ __forceinline__ float* V(float* base) const { return base + row(); }
  __device__ __forceinline__ float* CK(float* base, int k) const { return base + ((size_t)c * P.maxd + k) * ld; }

  // Per-element products and each thread's partial sums are FP32 (numpyro's dtype); the
  // partials are summed across the group as float-float pairs and used as FP64.  GB300 issues
  // FP64 at a small fraction of the FP32 rate, so per-element FP64 (or FP64 reductions run by
  // every thread of the group) would dominate the leaves of large-D chains.
  // Element loops are blocked by UB: a thread issues the loads of UB of its elements before any
  // store, so one memory round trip covers UB elements (stores to one chain buffer and loads
  // from another could otherwise not be reordered by the compiler).  Each thread only ever
  // touches its own elements d = tid + k * NT, in increasing d, so results do not depend on UB.
  // A warp per chain (the hierarchical family, J up to a few hundred) gains from 8 loads in
  // flight; a CTA per chain (T = 4096: 16 elements per thread) loses occupancy with 8 and keeps 4.
  static constexpr int UB = NT == 32 ? 8 : 4;

  // 0.5 * r . (M^-1 r)
  __device__ double kinetic(const float* r) {
    const float* mi = V(P.s.inverse_mass_matrix);
    float acc = 0.0f;
    for (int d0 = g.tid; d0 < D; d0 += UB * NT) {
      float rr[UB], mm[UB];
#pragma unroll
      for (int k = 0; k < UB; ++k) {
        const int d = d0 + k * NT;
        rr[k] = (d < D) ? r[d] : 0.0f;
        mm[k] = (d < D) ? mi[d] : 0.0f;
      }
#pragma unroll
      for (int k = 0; k < UB; ++k)
        if (d0 + k * NT < D) acc = fmaf(mm[k] * rr[k], rr[k], acc);
    }
    return 0.5 * ff_value(g.sumff(ff_from(acc), red));
  }

  // _is_turning: v_l . (rs - (r_l + r_r)/2) <= 0 or v_r . (...) <= 0, with v = M^-1 r;
  // the subtree sum rs - rs_minus + rs_plus of _is_iterative_turning when rs_minus is given
  __device__ bool is_turning(const float* rl, const float* rr, const float* rs, const float* rs_minus,
                             const float* rs_plus) {
    if (DM) return is_turning_dense(rl, rr, rs, rs_minus, rs_plus);
    const float* mi = V(P.s.inverse_mass_matrix);
    float ax = 0.0f, ay = 0.0f;
    for (int d0 = g.tid; d0 < D; d0 += UB * NT) {
      float sv[UB], av[UB], bv[UB], mv[UB];
#pragma unroll
      for (int k = 0; k < UB; ++k) {
        const int d = d0 + k * NT;
        const bool in = d < D;
        sv[k] = in ? rs[d] : 0.0f;
        if (rs_minus) sv[k] = in ? (sv[k] - rs_minus[d]) + rs_plus[d] : 0.0f;
        av[k] = in ? rl[d] : 0.0f;
        bv[k] = in ? rr[d] : 0.0f;
        mv[k] = in ? mi[d] : 0.0f;
      }
#pragma unroll
      for (int k = 0; k < UB; ++k) {
        if (d0 + k * NT >= D) continue;
        const float s = sv[k] - 0.5f * (av[k] + bv[k]);
        ax = fmaf(mv[k] * av[k], s, ax);
        ay = fmaf(mv[k] * bv[k], s, ay);
      }
    }
    FF tx = ff_from(ax), ty = ff_from(ay);
    g.sum2ff(tx, ty, red);
    return ff_le0(tx) || ff_le0(ty);
  }

  __device__ void copy(float* dst, const float* src) {
    for (int d0 = g.tid; d0 < D; d0 += UB * NT) {
      float v[UB];
#pragma unroll
      for (int k = 0; k < UB; ++k) v[k] = (d0 + k * NT < D) ? src[d0 + k * NT] : 0.0f;
#pragma unroll
      for (int k = 0; k < UB; ++k)
        if (d0 + k * NT < D) dst[d0 + k * NT] = v[k];
    }
  }

  // ----------------------------------------------------------- dense mass matrix helpers
  // [D][D] matrices of this chain (row stride ld)
  __device__ __forceinline__ float* MX(float* base) const { return base + (size_t)c * ld * ld; }
  // use(d, (A x)_d) for this thread's elements d, A symmetric (read by columns: A[j][d]); x is
  // read in full, so the group must have synchronised after writing it
  template <typename F>
  __device__ void sym_matvec(const float* A, const float* x, F&& use) {
    for (int d0 = g.tid; d0 < D; d0 += UB * NT) {
      float acc[UB] = {};
      for (int j = 0; j < D; ++j) {
        const float xj = x[j];
        const float* Aj = A + (size_t)j * ld + d0;
#pragma unroll
        for (int k = 0; k < UB; ++k)
          if (d0 + k * NT < D) acc[k] = fmaf(Aj[k * NT], xj, acc[k]);
      }
#pragma unroll
      for (int k = 0; k < UB; ++k)
        if (d0 + k * NT < D) use(d0 + k * NT, acc[k]);
    }
  }
  // 0.5 r . (M^-1 r) with a dense M^-1 (euclidean_kinetic_energy, hmc_util.py:1183-1200)
  __device__ double kinetic_dense(const float* r) {
    g.sync();
    float acc = 0.0f;
    sym_matvec(MX(P.s.inverse_mass_matrix), r, [&](int d, float v) { acc = fmaf(v, r[d], acc); });
    return 0.5 * ff_value(g.sumff(ff_from(acc), red));
  }
  // _is_turning with a dense M^-1: v_l . s = r_l . (M^-1 s) as M^-1 is symmetric
  __device__ bool is_turning_dense(const float* rl, const float* rr, const float* rs, const float* rs_minus,
                                   const float* rs_plus) {
    float* sv = V(P.e.tmp);
    for (int d = g.tid; d < D; d += NT) {
      float s_ = rs[d];
      if (rs_minus) s_ = (s_ - rs_minus[d]) + rs_plus[d];
      sv[d] = s_ - 0.5f * (rl[d] + rr[d]);
    }
    g.sync();
    float ax = 0.0f, ay = 0.0f;
    sym_matvec(MX(P.s.inverse_mass_matrix), sv, [&](int d, float w) {
      ax = fmaf(rl[d], w, ax);
      ay = fmaf(rr[d], w, ay);
    });
    FF tx = ff_from(ax), ty = ff_from(ay);
    g.sum2ff(tx, ty, red);  // also keeps every thread's reads of sv before the next write
    return ff_le0(tx) || ff_le0(ty);
  }
  // r = S eps (momentum_generator, hmc.py:92-110) with eps in the scratch row; S row-major
  __device__ void dense_momentum(const float* Smat, float* r_out) {
    const float* eps = V(P.e.tmp);
    for (int i = g.tid; i < D; i += NT) {
      const float* Si = Smat + (size_t)i * ld;
      float acc = 0.0f;
      for (int j = 0; j < D; ++j) acc = fmaf(Si[j], eps[j], acc);
      r_out[i] = acc;
    }
  }

  // ----------------------------------------------------------- leapfrog halves
  // first half-kick + drift from the frontier on side `right`; writes Q
  __device__ void leaf_prepare(bool right, float eps) {
    float* z = (right ? z_r_() : z_l_());
    float* r = (right ? r_r_() : r_l_());
    const float* gr = (right ? g_r_() : g_l_());
    const float* mi = V(P.s.inverse_mass_matrix);
    float* q = Q_();
    if (DM) {  // r_half = r - eps/2 g; z += eps M^-1 r_half
      for (int d = g.tid; d < D; d += NT) r[d] = r[d] - 0.5f * eps * gr[d];
      g.sync();
      sym_matvec(MX(P.s.inverse_mass_matrix), r, [&](int d, float v) {
        const float zn = z[d] + eps * v;
        z[d] = zn;
        put_q(q, d, zn);
      });
      return;
    }
    for (int d0 = g.tid; d0 < D; d0 += UB * NT) {
      float zz[UB], rr[UB], gg[UB], mm[UB];
#pragma unroll
      for (int k = 0; k < UB; ++k) {
        const int d = d0 + k * NT;
        const bool in = d < D;
        zz[k] = in ? z[d] : 0.0f;
        rr[k] = in ? r[d] : 0.0f;
        gg[k] = in ? gr[d] : 0.0f;
        mm[k] = in ? mi[d] : 0.0f;
      }
#pragma unroll
      for (int k = 0; k < UB; ++k) {
        const int d = d0 + k * NT;
        if (d >= D) continue;
        float rh = rr[k] - 0.5f * eps * gg[k];
        float zn = zz[k] + eps * (mm[k] * rh);
        r[d] = rh;
        z[d] = zn;
        put_q(q, d, zn);
      }
    }
  }
  // second half-kick with the new gradient; returns K(r_new)
  __device__ double leaf_finish(bool right, float eps) {
    float* r = (right ? r_r_() : r_l_());
    float* gr = (right ? g_r_() : g_l_());
    const float* G = G_();
    const float* mi = V(P.s.inverse_mass_matrix);
    if (DM) {
      for (int d = g.tid; d < D; d += NT) {
        const float gn = G[d];
        r[d] = r[d] - 0.5f * eps * gn;
        gr[d] = gn;
      }
      return kinetic_dense(r);
    }
    float acc = 0.0f;  // kinetic energy of the new momentum, as kinetic()
    for (int d0 = g.tid; d0 < D; d0 += UB * NT) {
      float gn[UB], rr[UB], mm[UB];
#pragma unroll
      for (int k = 0; k < UB; ++k) {
        const int d = d0 + k * NT;
        const bool in = d < D;
        gn[k] = in ? G[d] : 0.0f;
        rr[k] = in ? r[d] : 0.0f;
        mm[k] = in ? mi[d] : 0.0f;
      }
#pragma unroll
      for (int k = 0; k < UB; ++k) {
        const int d = d0 + k * NT;
        if (d >= D) continue;
        const float rn = rr[k] - 0.5f * eps * gn[k];
        r[d] = rn;
        gr[d] = gn[k];
        acc = fmaf(mm[k] * rn, rn, acc);
      }
    }
    return 0.5 * ff_value(g.sumff(ff_from(acc), red));
  }

  __device__ float signed_step() const { return ctl.dir ? ctl.step : -ctl.step; }

  // ----------------------------------------------------------- transitions
  __device__ void start_transition() {
    uint32_t n = P.s.rng_key[2 * c + 1];
    uint32_t chain_id = P.s.rng_key[2 * c];
    const float* ms = V(P.s.mass_matrix_sqrt);
    const float* z = V(P.s.z);
    const float* gz = V(P.s.z_grad);
    float *zl = z_l_(), *zr = z_r_(), *zp = z_p_();
    float *rl = r_l_(), *rr = r_r_(), *rs = rsum_();
    float *gl = g_l_(), *grr = g_r_(), *gp = g_p_();
    float kin = 0.0f;
    const float* mi = V(P.s.inverse_mass_matrix);
    double kin_dense = 0.0;
    if (DM) {  // eps -> scratch; r = S eps; K = r . (M^-1 r) / 2
      float* eps = V(P.e.tmp);
      for (int d = g.tid; d < D; d += NT) {
        eps[d] = normal_at(P.seed, chain_id, n, P_MOMENTUM, d, 0);
        zl[d] = z[d]; zr[d] = z[d]; zp[d] = z[d];
        gl[d] = gz[d]; grr[d] = gz[d]; gp[d] = gz[d];
      }
      g.sync();
      dense_momentum(MX(P.s.mass_matrix_sqrt), rl);
      for (int d = g.tid; d < D; d += NT) {
        rr[d] = rl[d];
        rs[d] = rl[d];
      }
      kin_dense = kinetic_dense(rl);
    }
    for (int d0 = g.tid; d0 < D && !DM; d0 += UB * NT) {
      float msv[UB], miv[UB], zv[UB], gv[UB];
#pragma unroll
      for (int k = 0; k < UB; ++k) {
        const int d = d0 + k * NT;
        const bool in = d < D;
        msv[k] = in ? ms[d] : 0.0f;
        miv[k] = in ? mi[d] : 0.0f;
        zv[k] = in ? z[d] : 0.0f;
        gv[k] = in ? gz[d] : 0.0f;
      }
#pragma unroll
      for (int k = 0; k < UB; ++k) {
        const int d = d0 + k * NT;
        if (d >= D) continue;
        float r = msv[k] * normal_at(P.seed, chain_id, n, P_MOMENTUM, d, 0);
        kin = fmaf(miv[k] * r, r, kin);
        zl[d] = zv[k]; zr[d] = zv[k]; zp[d] = zv[k];
        gl[d] = gv[k]; grr[d] = gv[k]; gp[d] = gv[k];
        rl[d] = r; rr[d] = r; rs[d] = r;
      }
    }
    const double kin0 = DM ? kin_dense : 0.5 * ff_value(g.sumff(ff_from(kin), red));
    int i = P.s.i[c];
    double pe = P.s.potential_energy[c];
    ctl.energy0 = pe + kin0;
    ctl.step = P.s.step_size[c];
    ctl.depth = 0;
    ctl.tree_w = 0.0;
    ctl.tree_turning = 0;
    ctl.tree_div = 0;
    ctl.tree_acc = 0.0;
    ctl.num_prop = 0;
    ctl.pe_p = pe;
    ctl.energy_p = ctl.energy0;
    ctl.max_depth_cur = (i < P.num_warmup) ? P.mtd_warmup : P.mtd;
    if (P.algo == 1) {  // fixed-length HMC, hmc.py:364-414
      int L;
      if (P.fixed_steps > 0) {
        L = P.fixed_steps;
      } else {
        L = (int)ceil(P.traj_len / (double)ctl.step);
      }
      if (L < 1) L = 1;
      if (P.traj_len > 0.0) ctl.step = (float)(P.traj_len / (double)L);
      ctl.hmc_left = L;
      ctl.hmc_total = L;
      ctl.dir = 1;
    }
  }

  __device__ void start_subtree() {
    uint32_t n = P.s.rng_key[2 * c + 1];
    uint32_t chain_id = P.s.rng_key[2 * c];
    uint4 w = draw(P.seed, chain_id, n, P_DOUBLING, (uint32_t)ctl.depth, 0);
    ctl.dir = u01f(w.x) < 0.5f ? 1 : 0;
    ctl.sub_num = 0;
    ctl.sub_div = 0;
    ctl.sub_turning = 0;
    leaf_prepare(ctl.dir, signed_step());
    ctl.phase = PH_LEAF;
  }

  // a leaf's gradient has arrived: _build_basetree + uniform combine + checkpoints
  __device__ void finish_leaf() {
    uint32_t n = P.s.rng_key[2 * c + 1];
    uint32_t chain_id = P.s.rng_key[2 * c];
    bool right = ctl.dir;
    double kin = leaf_finish(right, signed_step());
    double pe = P.e.PE[c];
    double e_new = pe + kin;
    double dE = e_new - ctl.energy0;
    if (isnan(dE)) dE = INFINITY;
    double w = -dE;
    int div = dE > P.max_dE;
    double acc = (double)exp_min1_f(-dE);
    const float* zf = (right ? z_r_() : z_l_());
    const float* rf = (right ? r_r_() : r_l_());
    const float* gf = (right ? g_r_() : g_l_());
    float* zsp = z_sp_();
    float* gsp = g_sp_();
    float* rss = rsum_sub_();
    int leaf_idx = ctl.sub_num;
    if (leaf_idx == 0) {
      for (int d0 = g.tid; d0 < D; d0 += UB * NT) {
        float zv[UB], gv[UB], rv[UB];
#pragma unroll
        for (int k = 0; k < UB; ++k) {
          const int d = d0 + k * NT;
          const bool in = d < D;
          zv[k] = in ? zf[d] : 0.0f;
          gv[k] = in ? gf[d] : 0.0f;
          rv[k] = in ? rf[d] : 0.0f;
        }
#pragma unroll
        for (int k = 0; k < UB; ++k) {
          const int d = d0 + k * NT;
          if (d >= D) continue;
          zsp[d] = zv[k];
          gsp[d] = gv[k];
          rss[d] = rv[k];
        }
      }
      ctl.sub_w = w;
      ctl.pe_sp = pe;
      ctl.energy_sp = e_new;
      ctl.sub_acc = acc;
    } else {
      const float p = sigmoid_f(w - ctl.sub_w);
      uint4 u = draw(P.seed, chain_id, n, P_LEAF, (uint32_t)ctl.depth, (uint32_t)leaf_idx);
      bool take = u01f(u.x) < p;
      for (int d0 = g.tid; d0 < D; d0 += UB * NT) {
        float zv[UB], gv[UB], rv[UB], sv[UB];
#pragma unroll
        for (int k = 0; k < UB; ++k) {
          const int d = d0 + k * NT;
          const bool in = d < D;
          zv[k] = (in && take) ? zf[d] : 0.0f;
          gv[k] = (in && take) ? gf[d] : 0.0f;
          rv[k] = in ? rf[d] : 0.0f;
          sv[k] = in ? rss[d] : 0.0f;
        }
#pragma unroll
        for (int k = 0; k < UB; ++k) {
          const int d = d0 + k * NT;
          if (d >= D) continue;
          if (take) {
            zsp[d] = zv[k];
            gsp[d] = gv[k];
          }
          rss[d] = sv[k] + rv[k];
        }
      }
      if (take) {
        ctl.pe_sp = pe;
        ctl.energy_sp = e_new;
      }
      ctl.sub_w = logaddexp_mixed(ctl.sub_w, w);
      ctl.sub_acc += acc;
    }
    ctl.sub_div = div;
    ctl.sub_num = leaf_idx + 1;
    // checkpoints (hmc_util.py:1034-1047)
    int idx_max = __popc((unsigned)(leaf_idx >> 1));
    int num_sub = __popc((unsigned)((~leaf_idx & (leaf_idx + 1)) - 1));
    int idx_min = idx_max - num_sub + 1;
    if ((leaf_idx & 1) == 0) {
      copy(CK(P.e.r_ck, idx_max), rf);
      copy(CK(P.e.rs_ck, idx_max), rss);
    }
    g.sync();
    bool turning = false;
    for (int k = idx_max; k >= idx_min && !turning; --k) {
      // subtree r_sum = r_sum - r_sum_ckpts[k] + r_ckpts[k]; left = r_ckpts[k], right = r
      turning = is_turning(CK(P.e.r_ck, k), rf, rss, CK(P.e.rs_ck, k), CK(P.e.r_ck, k));
    }
    ctl.sub_turning = turning;
  }

  // subtree done: biased combine into the tree (hmc_util.py:936-938 -> :767-848)
  __device__ void combine_subtree() {
    uint32_t n = P.s.rng_key[2 * c + 1];
    uint32_t chain_id = P.s.rng_key[2 * c];
    float* rs = rsum_();
    const float* rss = rsum_sub_();
    for (int d0 = g.tid; d0 < D; d0 += UB * NT) {
      float a[UB], b[UB];
#pragma unroll
      for (int k = 0; k < UB; ++k) {
        const int d = d0 + k * NT;
        a[k] = (d < D) ? rs[d] : 0.0f;
        b[k] = (d < D) ? rss[d] : 0.0f;
      }
#pragma unroll
      for (int k = 0; k < UB; ++k)
        if (d0 + k * NT < D) rs[d0 + k * NT] = a[k] + b[k];
    }
    g.sync();
    float p;
    if (ctl.sub_turning || ctl.sub_div) {
      p = 0.0f;
    } else {
      p = exp_min1_f(ctl.sub_w - ctl.tree_w);
    }
    bool turning = ctl.sub_turning;
    if (!turning) turning = is_turning(r_l_(), r_r_(), rs, nullptr, nullptr);
    uint4 u = draw(P.seed, chain_id, n, P_DOUBLING, (uint32_t)ctl.depth, 0);
    bool take = u01f(u.y) < p;
    if (take) {
      copy(z_p_(), z_sp_());
      copy(g_p_(), g_sp_());
      ctl.pe_p = ctl.pe_sp;
      ctl.energy_p = ctl.energy_sp;
    }
    ctl.depth += 1;
    ctl.tree_w = logaddexp_mixed(ctl.tree_w, ctl.sub_w);
    ctl.tree_div = ctl.sub_div;
    ctl.tree_acc += ctl.sub_acc;
    ctl.num_prop += ctl.sub_num;
    ctl.tree_turning = turning;
  }

  // ----------------------------------------------------------- adaptation
  // returns true if a heuristic step-size search was started (pending)
  __device__ bool adapt(int t, double accept_prob) {
    double* ss = P.s.ss_state + 5 * (size_t)c;
    // Every thread of the group reads the chain's adaptation scalars before thread 0 updates
    // them (with a CTA per chain, warps run apart and would otherwise see a mix of old and
    // new values and take different branches).
    float step = P.s.step_size[c];
    double x_t = ss[0], x_avg = ss[1], g_avg = ss[2], tt = ss[3];
    const double prox = ss[4];
    int widx = P.s.window_idx[c];
    int nn = P.s.mm_n[c];
    g.sync();
    if (P.adapt_step) {  // dual_averaging.update_fn, t0=10, kappa=0.75, gamma=0.05
      double g_ = (double)P.target_accept - accept_prob;
      // the state stays FP64; the factors 1/(t+t0), sqrt(t)/gamma and t^-kappa of the integer
      // count t are formed with one FP64 division and FP32 sqrt/pow (correctly rounded / 1 ulp)
      tt += 1.0;
      const double inv_t = 1.0 / (tt + 10.0);
      g_avg = (1.0 - inv_t) * g_avg + g_ * inv_t;
      x_t = prox - 20.0 * (double)sqrtf((float)tt) * g_avg;
      const double wt = (double)powf((float)tt, -0.75f);
      x_avg = (1.0 - wt) * x_avg + wt * x_t;
      if (g.tid == 0) {
        ss[0] = x_t; ss[1] = x_avg; ss[2] = g_avg; ss[3] = tt;
      }
      float sf = expf((float)((t == P.num_warmup - 1) ? x_avg : x_t));
      if (!(sf >= FLT32_TINY)) sf = FLT32_TINY;  // also maps NaN to tiny
      if (sf > FLT32_MAX) sf = FLT32_MAX;
      step = sf;
    }
    bool middle = (0 < widx) && (widx < P.num_windows - 1);
    const float* z = V(P.s.z);
    double* mean = P.s.mm_mean + row();
    double* m2 = DM ? P.s.mm_m2 + (size_t)c * ld * ld : P.s.mm_m2 + row();
    if (P.adapt_mass && middle) {  // welford update_fn
      nn += 1;
      const double inv_n = 1.0 / (double)nn;
      if (DM) {  // m2 += outer(delta_post, delta_pre)
        double* dpost = P.e.tmpd + (size_t)c * 2 * ld;
        double* dpre = dpost + ld;
        for (int d = g.tid; d < D; d += NT) {
          const double x = (double)z[d];
          const double dp = x - mean[d];
          const double mnew = mean[d] + dp * inv_n;
          mean[d] = mnew;
          dpre[d] = dp;
          dpost[d] = x - mnew;
        }
        g.sync();
        for (int j = g.tid; j < D; j += NT) {
          const double pj = dpre[j];
          for (int i = 0; i < D; ++i) m2[(size_t)i * ld + j] += dpost[i] * pj;
        }
      } else {
        for (int d = g.tid; d < D; d += NT) {
          double x = (double)z[d];
          double dpre = x - mean[d];
          double mnew = mean[d] + dpre * inv_n;
          mean[d] = mnew;
          m2[d] += dpre * (x - mnew);
        }
      }
      if (g.tid == 0) P.s.mm_n[c] = nn;
    }
    bool at_end = (widx < P.num_windows) && (t == P.window_end[widx]);
    if (at_end) widx += 1;
    if (g.tid == 0) P.s.window_idx[c] = widx;
    bool started = false;
    if (at_end && middle) {
      if (DM && P.adapt_mass) {  // welford final_fn (dense) + Stan regularisation
        const double a = P.regularize ? (double)nn / (nn + 5.0) : 1.0;
        const double shrink = P.regularize ? 1e-3 * (5.0 / (nn + 5.0)) : 0.0;
        const double inv_nm1 = 1.0 / (double)(nn - 1);
        g.sync();
        const int32_t* blk = P.mass_block;  // block-structured: entries across blocks are zero
        for (int j = g.tid; j < D; j += NT)
          for (int i = 0; i < D; ++i) {
            const size_t o = (size_t)i * ld + j;
            const bool keep = !blk || i == j || (blk[i] >= 0 && blk[i] == blk[j]);
            m2[o] = keep ? a * (m2[o] * inv_nm1) + (i == j ? shrink : 0.0) : 0.0;
          }
        dense_factor(g, m2, D, ld, MX(P.s.inverse_mass_matrix), MX(P.s.mass_matrix_sqrt),
                     MX(P.s.mass_matrix_sqrt_inv));
        for (int d = g.tid; d < D; d += NT) mean[d] = 0.0;
        if (g.tid == 0) P.s.mm_n[c] = 0;
      } else if (P.adapt_mass) {  // welford final_fn + Stan regularisation (nn counts this draw)
        float* inv = V(P.s.inverse_mass_matrix);
        float* sq = V(P.s.mass_matrix_sqrt);
        float* sqi = V(P.s.mass_matrix_sqrt_inv);
        for (int d = g.tid; d < D; d += NT) {
          double cov = m2[d] / (double)(nn - 1);
          if (P.regularize) cov = ((double)nn / (nn + 5.0)) * cov + 1e-3 * (5.0 / (nn + 5.0));
          float covf = (float)cov;
          float ti = sqrtf(covf);
          inv[d] = covf;
          sqi[d] = ti;
          sq[d] = 1.0f / ti;
          mean[d] = 0.0;
          m2[d] = 0.0;
        }
        if (g.tid == 0) P.s.mm_n[c] = 0;
      }
      if (P.adapt_step) {
        if (P.heuristic) {
          if (g.tid == 0) P.s.step_size[c] = step;
          g.sync();
          heur_begin(HC_WINDOW, (uint32_t)t);
          started = true;
        } else if (g.tid == 0) {
          ss[0] = 0.0; ss[1] = 0.0; ss[2] = 0.0; ss[3] = 0.0;
          ss[4] = log(10.0) + log((double)step);
        }
      }
    }
    if (!started && g.tid == 0) P.s.step_size[c] = step;
    g.sync();
    return started;
  }

  // ----------------------------------------------------------- heuristic step size
  // find_reasonable_step_size (hmc_util.py:314-384).  The trial momentum is
  // generated from the inverse mass matrix, as the reference does at :356.
  __device__ void heur_begin(int ctx, uint32_t n_ctx) {
    ctl.heur_ctx = ctx;
    ctl.heur_step = (double)P.s.step_size[c];
    ctl.heur_dir = 0;
    ctl.heur_last = 0;
    ctl.heur_trial = 0;
    ctl.hmc_total = (int)n_ctx;  // stream index of this search
    heur_prepare();
  }
  __device__ void heur_prepare() {
    uint32_t chain_id = P.s.rng_key[2 * c];
    ctl.heur_step = exp2((double)ctl.heur_dir) * ctl.heur_step;
    float eps = (float)ctl.heur_step;
    const float* mi = V(P.s.inverse_mass_matrix);
    const float* z = V(P.s.z);
    const float* gz = V(P.s.z_grad);
    float* r0 = r_l_();
    float* rh = r_r_();
    float* q = Q_();
    if (DM) {
      // the trial momentum is M^-1 eps, as momentum_generator(z, inverse_mass_matrix, key) at
      // hmc_util.py:356 (the dense inverse mass matrix stands in for the square root there)
      float* epsv = V(P.e.tmp);
      for (int d = g.tid; d < D; d += NT)
        epsv[d] = normal_at(P.seed, chain_id, (uint32_t)ctl.hmc_total, P_HEURISTIC, d, (uint32_t)ctl.heur_trial);
      g.sync();
      sym_matvec(MX(P.s.inverse_mass_matrix), epsv, [&](int d, float v) {
        r0[d] = v;
        rh[d] = v - 0.5f * eps * gz[d];
      });
      const double k0 = kinetic_dense(r0);  // synchronises after r0 and rh were written
      sym_matvec(MX(P.s.inverse_mass_matrix), rh, [&](int d, float v) { put_q(q, d, z[d] + eps * v); });
      ctl.heur_e0 = P.s.potential_energy[c] + k0;
      ctl.phase = PH_HEUR;
      return;
    }
    float kin = 0.0f;
    for (int d = g.tid; d < D; d += NT) {
      float r = mi[d] * normal_at(P.seed, chain_id, (uint32_t)ctl.hmc_total, P_HEURISTIC, d,
                                  (uint32_t)ctl.heur_trial);
      kin = fmaf(mi[d] * r, r, kin);
      r0[d] = r;
      float h = r - 0.5f * eps * gz[d];
      rh[d] = h;
      put_q(q, d, z[d] + eps * (mi[d] * h));
    }
    ctl.heur_e0 = P.s.potential_energy[c] + 0.5 * ff_value(g.sumff(ff_from(kin), red));
    ctl.phase = PH_HEUR;
  }
  // returns true when the search is over (step size in ctl.heur_step)
  __device__ bool heur_finish() {
    float eps = (float)ctl.heur_step;
    const float* mi = V(P.s.inverse_mass_matrix);
    const float* G = G_();
    const float* rh = r_r_();
    double e_new;
    if (DM) {
      float* rn = r_r_();  // r_new overwrites r_half in place
      for (int d = g.tid; d < D; d += NT) rn[d] = rn[d] - 0.5f * eps * G[d];
      e_new = P.e.PE[c] + kinetic_dense(rn);
    } else {
      float kin = 0.0f;
      for (int d = g.tid; d < D; d += NT) {
        float rn = rh[d] - 0.5f * eps * G[d];
        kin = fmaf(mi[d] * rn, rn, kin);
      }
      e_new = P.e.PE[c] + 0.5 * ff_value(g.sumff(ff_from(kin), red));
    }
    double dE = e_new - ctl.heur_e0;
    int dir_new = (log(0.8) < -dE) ? 1 : -1;
    ctl.heur_last = ctl.heur_dir;
    ctl.heur_dir = dir_new;
    ctl.heur_trial += 1;
    double s = ctl.heur_step;
    bool not_small = (s > (double)FLT32_TINY) || (ctl.heur_dir >= 0);
    bool not_large = (s < (double)FLT32_MAX) || (ctl.heur_dir <= 0);
    bool cont = not_small && not_large && ((ctl.heur_last == 0) || (ctl.heur_dir == ctl.heur_last));
    if (cont && ctl.heur_trial < 4096) {
      heur_prepare();
      return false;
    }
    return true;
  }
  __device__ void heur_done() {
    float step = (float)ctl.heur_step;
    double* ss = P.s.ss_state + 5 * (size_t)c;
    if (g.tid == 0) {
      P.s.step_size[c] = step;
      ss[0] = 0.0; ss[1] = 0.0; ss[2] = 0.0; ss[3] = 0.0;
      ss[4] = (ctl.heur_ctx == HC_INIT) ? log(10.0 * (double)step) : log(10.0) + log((double)step);
    }
    g.sync();
  }

  // ----------------------------------------------------------- end of transition
  // returns true if the chain is now pending on a gradient (heuristic search)
  __device__ bool finish_transition(double pe_new, double energy_new, int num_steps, double accept_prob,
                                    int diverging, const float* znew, const float* gnew) {
    float* z = V(P.s.z);
    float* gz = V(P.s.z_grad);
    if (znew != z) {
      copy(z, znew);
      copy(gz, gnew);
    }
    const int i = P.s.i[c];  // read by every thread before thread 0 advances it
    g.sync();
    int j = ctl.iters_done;
    if (g.tid == 0) {
      P.s.potential_energy[c] = pe_new;
      P.s.energy[c] = energy_new;
      P.s.num_steps[c] = num_steps;
      P.s.accept_prob[c] = (float)accept_prob;
      P.s.diverging[c] = (uint8_t)diverging;
      int itr = i + 1;
      int nn = (i < P.num_warmup) ? itr : itr - P.num_warmup;
      float m = P.s.mean_accept_prob[c];
      P.s.mean_accept_prob[c] = m + ((float)accept_prob - m) / (float)nn;
      P.s.i[c] = itr;
      P.s.rng_key[2 * c + 1] += 1u;
    }
    // collection
    if (j >= P.collect_start && ((j - P.collect_start) % P.thinning) == 0) {
      int sidx = (j - P.collect_start) / P.thinning;
      if (sidx < P.num_collect) {
        size_t o = (size_t)c * P.num_collect + sidx;
        if (P.col.samples) {
          float* dst = P.col.samples + o * ld;
          copy(dst, znew);
        }
        if (g.tid == 0) {
          if (P.col.num_steps) P.col.num_steps[o] = num_steps;
          if (P.col.accept_prob) P.col.accept_prob[o] = (float)accept_prob;
          if (P.col.diverging) P.col.diverging[o] = (uint8_t)diverging;
          if (P.col.potential_energy) P.col.potential_energy[o] = pe_new;
        }
      }
    }
    g.sync();
    bool pending = false;
    if (i < P.num_warmup) pending = adapt(i, accept_prob);
    if (j >= P.collect_start && ((j - P.collect_start) % P.thinning) == 0 && !pending) {
      int sidx = (j - P.collect_start) / P.thinning;
      if (sidx < P.num_collect && P.col.step_size && g.tid == 0)
        P.col.step_size[(size_t)c * P.num_collect + sidx] = P.s.step_size[c];
    }
    ctl.iters_done = j + 1;
    ctl.iters_left -= 1;
    if (P.lockstep && g.tid == 0) atomicAdd(&P.done_count[j], 1);
    return pending;
  }

  // may a new transition start now?
  __device__ bool may_start() {
    if (ctl.iters_left <= 0) return false;
    if (!P.lockstep || ctl.iters_done == 0) return true;
    // Other chains raise the count concurrently: thread 0 reads it once and the group sum hands
    // that one reading to every thread, so all warps of a CTA-per-chain group decide alike.
    const int cnt = (g.tid == 0) ? *((volatile int32_t*)&P.done_count[ctl.iters_done - 1]) : 0;
    return g.sumff(ff_from((float)cnt), red).hi >= (float)P.C;  // counts <= 2^24 are exact
  }

  // ----------------------------------------------------------- driver
  __device__ void run() {
    bool need_start = false;
    switch (ctl.phase) {
      case PH_START:
        need_start = true;
        break;
      case PH_HEUR_START:
        heur_begin(HC_INIT, INIT_TRANSITION);
        return;
      case PH_HEUR:
        if (heur_finish()) {
          heur_done();
          if (ctl.heur_ctx == HC_INIT) {
            ctl.phase = PH_DONE;
            return;
          }
          need_start = true;  // window-end search finished: continue sampling
        } else {
          return;
        }
        break;
      case PH_WAIT:
        need_start = true;
        break;
      case PH_HMC: {
        double kin = leaf_finish(true, ctl.step);
        ctl.hmc_left -= 1;
        if (ctl.hmc_left > 0) {
          leaf_prepare(true, ctl.step);
          return;
        }
        // Metropolis correction (hmc.py:395-414)
        double pe = P.e.PE[c];
        double e_new = pe + kin;
        double dE = e_new - ctl.energy0;
        if (isnan(dE)) dE = INFINITY;
        double acc = (double)exp_min1_f(-dE);
        int div = dE > P.max_dE;
        uint32_t n = P.s.rng_key[2 * c + 1];
        uint32_t chain_id = P.s.rng_key[2 * c];
        uint4 u = draw(P.seed, chain_id, n, P_HMC_ACCEPT, 0, 0);
        bool take = u01f(u.x) < (float)acc;
        bool pend;
        if (take)
          pend = finish_transition(pe, e_new, ctl.hmc_total, acc, div, z_r_(), g_r_());
        else
          pend = finish_transition(P.s.potential_energy[c], ctl.energy0, ctl.hmc_total, acc, div, V(P.s.z),
                                   V(P.s.z_grad));
        if (pend) return;
        need_start = true;
        break;
      }
      case PH_LEAF: {
        finish_leaf();
        bool cont_sub = (ctl.sub_num < (1 << ctl.depth)) && !ctl.sub_turning && !ctl.sub_div;
        if (cont_sub) {
          leaf_prepare(ctl.dir, signed_step());
          return;
        }
        combine_subtree();
        bool cont_tree = (ctl.depth < ctl.max_depth_cur) && !ctl.tree_turning && !ctl.tree_div;
        if (cont_tree) {
          start_subtree();
          return;
        }
        double accept_prob = ctl.tree_acc / (double)ctl.num_prop;
        bool pend = finish_transition(ctl.pe_p, ctl.energy_p, ctl.num_prop, accept_prob, ctl.tree_div,
                                      z_p_(), g_p_());
        if (pend) return;
        need_start = true;
        break;
      }
      default:
        return;
    }
    if (need_start) {
      if (!may_start()) {
        ctl.phase = (ctl.iters_left > 0) ? PH_WAIT : PH_DONE;
        return;
      }
      start_transition();
      if (P.algo == 1) {
        leaf_prepare(true, ctl.step);
        ctl.phase = PH_HMC;
      } else {
        start_subtree();  // depth 0 < max_depth always holds for max_tree_depth >= 1
      }
    }
  }
};

// The parameter block lives in device memory (so captured CUDA graphs stay valid when the
// caller's buffers change between calls).  The state-machine kernels read its ~0.5 KB through
// hundreds of dependent field loads; a CTA stages it in shared memory once instead.
__device__ __forceinline__ const AdvParams& stage_params(const AdvParams* __restrict__ Pp, AdvParams* sp) {
  static_assert(sizeof(AdvParams) % 16 == 0, "AdvParams is copied as 16-byte words");
  const uint4* src = reinterpret_cast<const uint4*>(Pp);
  uint4* dst = reinterpret_cast<uint4*>(sp);
  for (int i = threadIdx.x; i < (int)(sizeof(AdvParams) / 16); i += blockDim.x) dst[i] = src[i];
  __syncthreads();
  return *sp;
}

template <int NT, bool DM>
__global__ void __launch_bounds__(256) advance_kernel(const AdvParams* __restrict__ Pp, int parity) {
  __shared__ double red[16];
  __shared__ __align__(16) AdvParams sp;
  const AdvParams& P = stage_params(Pp, &sp);
  int c;
  int tid;
  if (NT == 32) {
    c = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    tid = threadIdx.x & 31;
  } else {
    c = blockIdx.x;
    tid = threadIdx.x;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    P.counters[2 * (parity ^ 1)] = 0;
    P.counters[2 * (parity ^ 1) + 1] = 0;
  }
  int pending = 0, active = 0;
  if (NT == 32 && P.lrf_part_g && c < P.C) {
    // the tensor-core logistic potential of the previous tick ends here for the chains that queried it
    const int ph = P.e.ctl[c].phase;
    if (ph == PH_LEAF || ph == PH_HMC || ph == PH_HEUR)
      logreg_finish_warp(P.e.Q, c, P.C, P.D, P.D, P.lrf_row_groups, P.lrf_part_g, P.lrf_part_ll, P.lrf_lin,
                         P.lrf_inv_var, P.lrf_pe_const, P.e.PE, P.e.G, tid, P.lrf_split3, P.lrf_e_tanh != 0);
    __syncwarp();  // G and PE written by other lanes
  }
  if (NT == 256 && P.hsf_part_gb && c < P.C) {
    // the tensor-core horseshoe potential of the previous tick ends here for a chain that queried it
    const int ph = P.e.ctl[c].phase;
    if (ph == PH_LEAF || ph == PH_HMC || ph == PH_HEUR)
      horseshoe_finish_block(P.e.Q, c, P.D, P.hsf_P, P.hsf_N, P.hsf_part_gb, P.hsf_splits, P.hsf_ldg, P.C,
                             P.hsf_part_rr, P.hsf_ld_rr, P.hsf_mtiles, P.hsf_nc, P.e.PE, P.e.G, tid, red);
    __syncthreads();  // G and PE written by other threads
  }
  if (c < P.C) {
    Chain<NT, DM> ch{P, Group<NT>{tid}, red, c, P.e.chain_dim ? P.e.chain_dim[c] : P.D, P.D, P.e.ctl[c], nullptr};
    ch.run();
    if (tid == 0) {
      P.e.ctl[c] = ch.ctl;
      int ph = ch.ctl.phase;
      pending = (ph == PH_LEAF || ph == PH_HMC || ph == PH_HEUR);
      active = (ph != PH_DONE && ph != PH_IDLE);
    }
  }
  int np = __syncthreads_count(pending);
  if (NT == 256 && P.hsf_bs && np && c < P.C) {
    // the coefficients of the position this chain queries, as the GEMMs take them: beta (or
    // tau lambda unscaled_beta when non-centred) split into bf16 hi/mid/lo, split_beta_kernel's
    // arithmetic (Q is complete: the count above synchronised the CTA)
    const float* z = P.e.Q + (size_t)c * P.D;
    const int Pn = P.hsf_P;
    for (int k = tid; k < Pn; k += NT) {
      const float v = P.hsf_nc ? expf(z[Pn + 1] + z[k]) * z[Pn + 2 + k] : z[k];
      const __nv_bfloat16 hi = __float2bfloat16_rn(v);
      const float r1 = v - __bfloat162float(hi);
      const __nv_bfloat16 mid = __float2bfloat16_rn(r1);
      const __nv_bfloat16 lo = __float2bfloat16_rn(r1 - __bfloat162float(mid));
      const size_t i = (size_t)c * P.hsf_kp + k;
      P.hsf_bs[i] = __bfloat16_as_ushort(hi);
      P.hsf_bs[P.hsf_total + i] = __bfloat16_as_ushort(mid);
      P.hsf_bs[2 * P.hsf_total + i] = __bfloat16_as_ushort(lo);
    }
  }
  int na = __syncthreads_count(active);
  if (threadIdx.x == 0) {
    if (np) atomicAdd(&P.counters[2 * parity], np);
    if (na) atomicAdd(&P.counters[2 * parity + 1], na);
  }
}

// --------------------------------------------------------------------- init kernels
// init_to_uniform(radius=2) for chains whose flag is set; writes z into st.z and Q
__global__ void init_uniform_kernel(const AdvParams* __restrict__ Pp, int attempt, const int32_t* __restrict__ flag) {
  const AdvParams& P = *Pp;
  size_t total = (size_t)P.C * P.D;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
    int c = (int)(k / P.D), d = (int)(k % P.D);
    if (flag && !flag[c]) continue;
    int Dc = P.e.chain_dim ? P.e.chain_dim[c] : P.D;
    float v = 0.0f;
    if (d < Dc) v = -2.0f + 4.0f * uniform_at(P.seed, P.s.rng_key[2 * c], (uint32_t)attempt, P_INIT, d, 0);
    P.s.z[k] = v;
  }
}

// validity of (pe, grad) per chain: flag[c] = 1 when not finite; counts invalid
__global__ void check_valid_kernel(const AdvParams* __restrict__ Pp, int32_t* flag, int32_t* count) {
  const AdvParams& P = *Pp;
  int c = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  int lane = threadIdx.x & 31;
  if (c >= P.C) return;
  int Dc = P.e.chain_dim ? P.e.chain_dim[c] : P.D;
  bool ok = true;
  for (int d = lane; d < Dc; d += 32) ok &= isfinite(P.s.z_grad[(size_t)c * P.D + d]);
  ok = __all_sync(0xffffffffu, ok);
  ok = ok && isfinite(P.s.potential_energy[c]);
  if (lane == 0) {
    flag[c] = ok ? 0 : 1;
    if (!ok) atomicAdd(count, 1);
  }
}

// HMCState / HMCAdaptState initial values (hmc.py:193-362, hmc_util.py:552-594)
__global__ void init_state_kernel(const AdvParams* __restrict__ Pp, const float* __restrict__ inv_mass_init,
                                  float init_step) {
  const AdvParams& P = *Pp;
  size_t total = (size_t)P.C * P.D;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
    int c = (int)(k / P.D), d = (int)(k % P.D);
    int Dc = P.e.chain_dim ? P.e.chain_dim[c] : P.D;
    if (!P.dense) {  // dense mass matrices are set by init_dense_mass_kernel
      float inv = (d < Dc) ? (inv_mass_init ? inv_mass_init[k] : 1.0f) : 0.0f;
      float si = sqrtf(inv);
      P.s.inverse_mass_matrix[k] = inv;
      P.s.mass_matrix_sqrt_inv[k] = si;
      P.s.mass_matrix_sqrt[k] = (d < Dc) ? 1.0f / si : 0.0f;
      P.s.mm_m2[k] = 0.0;
    }
    P.s.mm_mean[k] = 0.0;
    if (d == 0) {
      P.s.i[c] = 0;
      P.s.num_steps[c] = 0;
      P.s.accept_prob[c] = 0.0f;
      P.s.mean_accept_prob[c] = 0.0f;
      P.s.diverging[c] = 0;
      P.s.step_size[c] = init_step;
      double* ss = P.s.ss_state + 5 * (size_t)c;
      ss[0] = 0.0; ss[1] = 0.0; ss[2] = 0.0; ss[3] = 0.0;
      ss[4] = log(10.0 * (double)init_step);
      P.s.mm_n[c] = 0;
      P.s.window_idx[c] = 0;
      P.s.rng_key[2 * c + 1] = 0u;
      P.s.energy[c] = P.s.potential_energy[c];
    }
  }
}

// Dense mass matrices at init (_initialize_mass_matrix, hmc_util.py:439-515): the identity, or
// the factorisation of a given [C][D][D] inverse mass matrix; zeroes the Welford m2.  A warp per
// chain.
__global__ void init_dense_mass_kernel(const AdvParams* __restrict__ Pp, const float* __restrict__ inv_mass_init) {
  const AdvParams& P = *Pp;
  const int c = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (c >= P.C) return;
  const int ld = P.D, Dc = P.e.chain_dim ? P.e.chain_dim[c] : P.D;
  const size_t base = (size_t)c * ld * ld;
  double* A = P.s.mm_m2 + base;
  float *inv = P.s.inverse_mass_matrix + base, *sq = P.s.mass_matrix_sqrt + base,
        *sqi = P.s.mass_matrix_sqrt_inv + base;
  for (size_t o = lane; o < (size_t)ld * ld; o += 32) {
    const int i = (int)(o / ld), j = (int)(o % ld);
    const float id = (i == j && i < Dc) ? 1.0f : 0.0f;
    inv[o] = id;
    sq[o] = id;
    sqi[o] = id;
    A[o] = (inv_mass_init && i < Dc && j < Dc) ? (double)inv_mass_init[base + o] : 0.0;
  }
  __syncwarp();
  if (inv_mass_init) dense_factor(Group<32>{lane}, A, Dc, ld, inv, sq, sqi);
}

__global__ void set_phase_kernel(const AdvParams* __restrict__ Pp, int phase, int iters) {
  const AdvParams& P = *Pp;
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= P.C) return;
  ChainCtl& k = P.e.ctl[c];
  k.phase = phase;
  k.iters_left = iters;
  k.iters_done = 0;
}

__global__ void set_rng_chain_kernel(uint32_t* rng_key, int C, int first_chain) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < C) {
    rng_key[2 * c] = (uint32_t)(first_chain + c);
    rng_key[2 * c + 1] = 0u;
  }
}

// --------------------------------------------------------------------- persistent engine
// For the hierarchical family the potential costs O(J) per gradient, so a launch
// per leapfrog step is pure overhead.  Each warp pops chains from a device work
// queue (ordered longest-first) and runs every requested transition of its chain --
// tree doubling, leaves, U-turn checks, adaptation, collection -- calling the
// warp-level potential inline between state-machine steps.  Chains never wait for
// one another; there is no grid-wide synchronisation and no spin-wait.
template <bool DM>
__global__ void __launch_bounds__(256) persistent_hier_kernel(const AdvParams* __restrict__ Pp, HierView hv,
                                                              int32_t* queue_head, const int32_t* __restrict__ order) {
  __shared__ __align__(16) AdvParams sp;
  const AdvParams& P = stage_params(Pp, &sp);
  const int lane = threadIdx.x & 31;
  for (;;) {
    int k = 0;
    if (lane == 0) k = atomicAdd(queue_head, 1);
    k = __shfl_sync(0xffffffffu, k, 0);
    if (k >= P.C) break;
    const int c = order ? order[k] : k;
    int m = c / hv.cpm;
    if (m >= hv.num_models) m = hv.num_models - 1;
    const int j0 = hv.off[m], J = hv.off[m + 1] - j0;
    Chain<32, DM> ch{P, Group<32>{lane}, nullptr, c, P.e.chain_dim ? P.e.chain_dim[c] : P.D, P.D, P.e.ctl[c], nullptr};
    ch.run();
    for (;;) {
      const int ph = ch.ctl.phase;
      if (!(ph == PH_LEAF || ph == PH_HMC || ph == PH_HEUR)) break;
      __syncwarp();  // Q written by other lanes
      hier_nc_potential_warp(P.e.Q + (size_t)c * P.D, P.e.G + (size_t)c * P.D, P.e.PE + c, J, hv.y + j0,
                             hv.sinv + j0, hv.cmodel[m], hv.inv_ms2, hv.inv_ts, lane);
      __syncwarp();  // G and PE written by other lanes
      ch.run();
    }
    if (lane == 0) P.e.ctl[c] = ch.ctl;
  }
}

// Stochastic volatility: one CTA per chain (D = T + 2 in the thousands).  Each CTA pops
// chains from the work queue and runs all their transitions with the CTA-level potential
// inline, so no leapfrog step costs a kernel launch or a host round trip.  Every thread
// carries the same ChainCtl (its decisions come from block-wide reductions and the
// counter-based stream), so the control flow is uniform across the CTA.
// ONCHIP keeps the chain's twelve tree vectors (frontiers, proposals, momentum sums) in dynamic
// shared memory (12 D floats): they live only within a transition, so nothing needs copying in
// or out.  The query/gradient rows, the U-turn checkpoints and the sampler state stay in global
// memory.
constexpr int SV_ONCHIP_VECS = 12;
template <bool ONCHIP>
__global__ void __launch_bounds__(256) persistent_sv_kernel(const AdvParams* __restrict__ Pp, SvView sv,
                                                            int32_t* queue_head) {
  __shared__ SvSmem<256> sm;
  __shared__ int next_chain;
  __shared__ __align__(16) AdvParams sp;
  extern __shared__ float onchip[];
  const AdvParams& P = stage_params(Pp, &sp);
  const int tid = threadIdx.x;
  for (;;) {
    if (tid == 0) next_chain = atomicAdd(queue_head, 1);
    __syncthreads();
    const int c = next_chain;
    __syncthreads();  // every thread has read next_chain before it is overwritten
    if (c >= P.C) break;
    Chain<256> ch{P, Group<256>{tid}, sm.red, c, P.D, P.D, P.e.ctl[c], nullptr};
    if (ONCHIP) ch.oc = onchip;  // SV_ONCHIP_VECS consecutive rows of D floats
    ch.run();
    float* q = P.e.Q + (size_t)c * P.D;
    float* gr = P.e.G + (size_t)c * P.D;
    for (;;) {
      const int ph = ch.ctl.phase;
      if (!(ph == PH_LEAF || ph == PH_HMC || ph == PH_HEUR)) break;
      __syncthreads();  // Q written by other threads
      if (sv.noncentred)
        sv_nc_potential_block<256>(q, gr, P.e.PE + c, sv.T, sv.ret, sv.s_rate, sv.nu_rate, tid, sm);
      else
        sv_potential_block<256>(q, gr, P.e.PE + c, sv.T, sv.ret, sv.s_rate, sv.nu_rate, tid, sm);
      __syncthreads();  // G and PE written by other threads
      ch.run();
    }
    if (tid == 0) P.e.ctl[c] = ch.ctl;
    __syncthreads();  // the on-chip rows are free for the next chain
  }
}

// --------------------------------------------------------------------- launchers
void launch_persistent_hier(const AdvParams* dP, const HierView& hv, int32_t* queue_head, const int32_t* order,
                            int C, bool dense, cudaStream_t st) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (dense)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, persistent_hier_kernel<true>, 256, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, persistent_hier_kernel<false>, 256, 0);
  if (per_sm < 1) per_sm = 1;
  int blocks = sms * per_sm;
  int need = (C + 7) / 8;  // never more warps than chains
  if (blocks > need) blocks = need;
  if (dense)
    persistent_hier_kernel<true><<<blocks, 256, 0, st>>>(dP, hv, queue_head, order);
  else
    persistent_hier_kernel<false><<<blocks, 256, 0, st>>>(dP, hv, queue_head, order);
}

void launch_persistent_sv(const AdvParams* dP, const SvView& sv, int32_t* queue_head, int C, int D,
                          cudaStream_t st) {
  int dev = 0, sms = 0, per_sm = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  // On-chip rows make each leaf about a quarter faster (T = 4096 on GB300), but at 12 D floats per
  // CTA they can cost resident chains (197 KB: one CTA per SM, against two with global rows).  They
  // are used only when every chain is resident either way.
  const size_t onchip = sizeof(float) * (size_t)SV_ONCHIP_VECS * D;
  bool use_onchip = onchip + sizeof(SvSmem<256>) + 64 <= (size_t)optin;
  if (use_onchip) {
    cudaFuncSetAttribute(persistent_sv_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)onchip);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, persistent_sv_kernel<true>, 256, onchip);
    if (per_sm < 1 || (int64_t)sms * per_sm < C) use_onchip = false;
  }
  if (!use_onchip) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, persistent_sv_kernel<false>, 256, 0);
  if (per_sm < 1) per_sm = 1;
  int blocks = sms * per_sm;
  if (blocks > C) blocks = C;
  if (use_onchip)
    persistent_sv_kernel<true><<<blocks, 256, onchip, st>>>(dP, sv, queue_head);
  else
    persistent_sv_kernel<false><<<blocks, 256, 0, st>>>(dP, sv, queue_head);
}

void launch_advance(const AdvParams* dP, int C, int D, bool cta_per_chain, bool dense, int parity, cudaStream_t st) {
  if (!cta_per_chain && D <= 1024) {
    int cpb = 8;
    if (dense)
      advance_kernel<32, true><<<(C + cpb - 1) / cpb, 32 * cpb, 0, st>>>(dP, parity);
    else
      advance_kernel<32, false><<<(C + cpb - 1) / cpb, 32 * cpb, 0, st>>>(dP, parity);
  } else {
    advance_kernel<256, false><<<C, 256, 0, st>>>(dP, parity);  // dense mass needs a warp per chain
  }
}

void launch_init_uniform(const AdvParams* dP, int C, int D, int attempt, const int32_t* flag, cudaStream_t st) {
  size_t total = (size_t)C * D;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  init_uniform_kernel<<<blocks, 256, 0, st>>>(dP, attempt, flag);
}

void launch_check_valid(const AdvParams* dP, int C, int32_t* flag, int32_t* count, cudaStream_t st) {
  check_valid_kernel<<<(C + 7) / 8, 256, 0, st>>>(dP, flag, count);
}

void launch_init_state(const AdvParams* dP, int C, int D, const float* inv_mass_init, float init_step,
                       cudaStream_t st) {
  size_t total = (size_t)C * D;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  init_state_kernel<<<blocks, 256, 0, st>>>(dP, inv_mass_init, init_step);
}

void launch_init_dense_mass(const AdvParams* dP, int C, const float* inv_mass_init, cudaStream_t st) {
  init_dense_mass_kernel<<<(C + 3) / 4, 128, 0, st>>>(dP, inv_mass_init);
}

void launch_set_phase(const AdvParams* dP, int C, int phase, int iters, cudaStream_t st) {
  set_phase_kernel<<<(C + 255) / 256, 256, 0, st>>>(dP, phase, iters);
}

void launch_set_rng_chain(uint32_t* rng_key, int C, int first_chain, cudaStream_t st) {
  set_rng_chain_kernel<<<(C + 255) / 256, 256, 0, st>>>(rng_key, C, first_chain);
}

__global__ void set_params_kernel(const AdvParams p, AdvParams* dst) {
  static_assert(sizeof(AdvParams) % 16 == 0, "AdvParams is copied as 16-byte words");
  const uint4* src = reinterpret_cast<const uint4*>(&p);
  uint4* d = reinterpret_cast<uint4*>(dst);
  for (int i = threadIdx.x; i < (int)(sizeof(AdvParams) / 16); i += blockDim.x) d[i] = src[i];
}

void launch_set_params(const AdvParams& p, AdvParams* dst, cudaStream_t st) {
  set_params_kernel<<<1, 32, 0, st>>>(p, dst);
}

__global__ void tick_condition_kernel(cudaGraphConditionalHandle handle, const int32_t* counters, int last,
                                      int32_t* iter, const int* tc_err, int32_t* err_word) {
  const int it = iter[0] + 1;
  iter[0] = it;
  const bool active = counters[2 * last + 1] != 0;
  const bool failed = tc_err != nullptr && *tc_err != 0;
  const bool over = it >= iter[1];
  if (active && (over || failed)) *err_word = 4;  // GBN_ERR_TIMEOUT
  cudaGraphSetConditional(handle, (active && !over && !failed) ? 1u : 0u);
}

void launch_tick_condition(unsigned long long cond_handle, const int32_t* counters, int last, int32_t* iter,
                           const int* tc_err, int32_t* err_word, cudaStream_t st) {
  tick_condition_kernel<<<1, 1, 0, st>>>((cudaGraphConditionalHandle)cond_handle, counters, last, iter, tc_err,
                                         err_word);
}

}  // namespace gbn
