// capi.cu -- the extern "C" boundary of libgbnuts (declared in include/gbnuts.h).
//
// Host-side engine: owns the model data and tree scratch, builds the Stan
// adaptation schedule (numpyro/infer/hmc_util.py:387-436), runs the
// validity-retrying initialisation (numpyro/infer/util.py:366-508) and drives
// the advance/potential "ticks" until every chain has finished the requested
// transitions.  No exception crosses the ABI; every entry point returns a
// status and records a message readable through gbn_last_error.
#include <cmath>
#include <cstdio>
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gbnuts.h"
#include "common.cuh"
#include "internal.h"

using namespace gbn;

struct gbn_handle_s {
  gbn_config cfg{};
  ModelDev m;
  int C = 0, D = 0, maxd = 1;
  EngineBufs e{};
  AdvParams hp{};
  AdvParams* dP = nullptr;
  int32_t* counters = nullptr;
  int32_t* h_counters = nullptr;  // pinned
  int32_t* done_count = nullptr;
  int done_cap = 0;
  int32_t* flags = nullptr;
  int32_t* err_word = nullptr;
  int32_t* window_end = nullptr;
  int persistent = 0;         // run gbn_run through the persistent engine
  bool cta_per_chain = false; // advance kernel: a CTA (not a warp) per chain
  int32_t* order = nullptr;   // persistent engine: chain queue order
  int num_windows = 0;
  int num_warmup = 0;
  int initialised = 0;
  std::string err;
  gbn_stats stats{};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<void*> allocs;
  // CUDA graph of one batch of ticks (advance + potential launches), replayed by tick_loop
  int use_graphs = 1;
  cudaStream_t cap_stream = nullptr;
  cudaGraphExec_t tick_graph = nullptr;
  void* graph_scratch = nullptr;  // potential scratch the graph was captured with
  std::string tuning;             // launch shapes chosen by the autotuner
  int64_t id = 0;                 // registry id (gbn_handle_id)
  double* vjp_pe = nullptr;       // potential values discarded by gbn_potential_vjp
  int vjp_cap = 0;
  // gbn_sample_async: a graph whose WHILE node repeats tick batches until no chain is active
  cudaGraphExec_t async_graph = nullptr;
  int32_t* async_iter = nullptr;  // [2]: loop iterations done, iteration budget
  void* async_scratch = nullptr;  // potential scratch the async graph was built with
  int fuse_tick = 1;              // GBN_FUSE_TICK=0: the tensor-core potentials' split and finish run unfused
};

// The tick engine fuses the tensor-core logistic potential's coefficient split and row-group finish
// into its advance kernel; the pointers (which a larger gbn_potential_and_grad call may reallocate)
// are refreshed before every upload of the parameter block.
static void refresh_fusion(gbn_handle h) {
  AdvParams& P = h->hp;
  P.lrf_part_g = nullptr;
  P.lrf_part_ll = nullptr;
  P.lrf_lin = nullptr;
  P.lrf_bsplit = nullptr;
  P.lrf_split3 = nullptr;
  P.lrf_e_tanh = 0;
  P.hsf_part_gb = nullptr;
  P.hsf_part_rr = nullptr;
  P.hsf_bs = nullptr;
  // the horseshoe's fused split and finish live in the CTA-per-chain state machine: with a latent
  // dimension <= 1024 the warp-per-chain kernel runs (launch_advance), and the separate kernels stay
  const bool cta_engine = h->cta_per_chain || h->D > 1024;
  if (h->fuse_tick && cta_engine && !h->persistent && h->m.family == GBN_FAMILY_HORSESHOE &&
      h->m.precision == GBN_PREC_BF16X3 && h->m.hs_tc && !horseshoe_tc_fusion(h->m, h->C, &P)) {
    P.hsf_part_gb = nullptr;
    P.hsf_bs = nullptr;
  }
  if (h->fuse_tick && !h->persistent && h->m.family == GBN_FAMILY_LOGREG && h->m.precision == GBN_PREC_BF16X3 &&
      h->m.tc && !logreg_tc_fusion(h->m, h->C, &P))
    P.lrf_part_g = nullptr;
}

static thread_local std::string g_last_error;

// Integer ids of live handles, for callers that can pass a handle only as a plain attribute (an
// XLA FFI handler bound through jax.ffi, which XLA may call from any thread).
static std::mutex g_handles_mu;
static std::map<int64_t, gbn_handle> g_handles;
static int64_t g_next_id = 1;

static int fail(gbn_handle h, int code, const std::string& msg) {
  g_last_error = msg;
  if (h) h->err = msg;
  return code;
}

static int cuda_fail(gbn_handle h, cudaError_t e, const char* what) {
  std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
  return fail(h, GBN_ERR_CUDA, msg);
}

template <typename T>
static cudaError_t dalloc(gbn_handle h, T** p, size_t count) {
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void**)p, sizeof(T) * count);
  if (e == cudaSuccess) {
    h->allocs.push_back((void*)*p);
    cudaMemset(*p, 0, sizeof(T) * count);
  }
  return e;
}

// Stan windows, numpyro/infer/hmc_util.py:387-436
static std::vector<int> adaptation_window_ends(int num_steps) {
  std::vector<int> ends;
  if (num_steps <= 0) return ends;
  if (num_steps < 20) {
    ends.push_back(num_steps - 1);
    return ends;
  }
  int start_buffer = 75, end_buffer = 50, init_window = 25;
  if (start_buffer + end_buffer + init_window > num_steps) {
    start_buffer = (int)(0.15 * num_steps);
    end_buffer = (int)(0.1 * num_steps);
    init_window = num_steps - start_buffer - end_buffer;
  }
  ends.push_back(start_buffer - 1);
  int end_window_start = num_steps - end_buffer;
  int next_size = init_window, next_start = start_buffer;
  while (next_start < end_window_start) {
    int cur_start = next_start, cur_size = next_size;
    if (3 * cur_size <= end_window_start - cur_start)
      next_size = 2 * cur_size;
    else
      cur_size = end_window_start - cur_start;
    next_start = cur_start + cur_size;
    ends.push_back(next_start - 1);
  }
  ends.push_back(num_steps - 1);
  return ends;
}

static void fill_state(AdvParams& P, const gbn_state* st) {
  P.s.i = st->i;
  P.s.z = st->z;
  P.s.z_grad = st->z_grad;
  P.s.potential_energy = st->potential_energy;
  P.s.energy = st->energy;
  P.s.num_steps = st->num_steps;
  P.s.accept_prob = st->accept_prob;
  P.s.mean_accept_prob = st->mean_accept_prob;
  P.s.diverging = st->diverging;
  P.s.step_size = st->step_size;
  P.s.inverse_mass_matrix = st->inverse_mass_matrix;
  P.s.mass_matrix_sqrt = st->mass_matrix_sqrt;
  P.s.mass_matrix_sqrt_inv = st->mass_matrix_sqrt_inv;
  P.s.ss_state = st->ss_state;
  P.s.mm_mean = st->mm_mean;
  P.s.mm_m2 = st->mm_m2;
  P.s.mm_n = st->mm_n;
  P.s.window_idx = st->window_idx;
  P.s.rng_key = st->rng_key;
}

static bool state_ok(const gbn_state* st) {
  return st && st->i && st->z && st->z_grad && st->potential_energy && st->energy && st->num_steps &&
         st->accept_prob && st->mean_accept_prob && st->diverging && st->step_size && st->inverse_mass_matrix &&
         st->mass_matrix_sqrt && st->mass_matrix_sqrt_inv && st->ss_state && st->mm_mean && st->mm_m2 &&
         st->mm_n && st->window_idx && st->rng_key;
}

extern "C" {

int gbn_abi_version(void) { return GBN_ABI_VERSION; }

int gbn_tc_available(void) {
  ModelDev probe;
  probe.family = GBN_FAMILY_LOGREG;
  probe.p = 1;
  probe.n = 1;
  return logreg_tc_supported(probe) ? 1 : 0;
}

const char* gbn_last_error(gbn_handle h) { return h ? h->err.c_str() : g_last_error.c_str(); }

int gbn_latent_dim(gbn_handle h, int32_t* dim) {
  if (!h || !dim) return fail(h, GBN_ERR_INVALID_ARG, "gbn_latent_dim: null argument");
  *dim = h->D;
  return GBN_OK;
}

int64_t gbn_handle_id(gbn_handle h) { return h ? h->id : 0; }

gbn_handle gbn_handle_from_id(int64_t id) {
  std::lock_guard<std::mutex> lock(g_handles_mu);
  auto it = g_handles.find(id);
  return it == g_handles.end() ? nullptr : it->second;
}

int gbn_destroy(gbn_handle h) {
  if (!h) return GBN_OK;
  if (h->id) {
    std::lock_guard<std::mutex> lock(g_handles_mu);
    g_handles.erase(h->id);
  }
  cudaDeviceSynchronize();
  if (h->m.tc) logreg_tc_free(h->m);
  if (h->m.hs_tc) horseshoe_tc_free(h->m);
  free_potential_scratch(h->m);
  for (void* p : h->allocs) cudaFree(p);
  if (h->h_counters) cudaFreeHost(h->h_counters);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->tick_graph) cudaGraphExecDestroy(h->tick_graph);
  if (h->async_graph) cudaGraphExecDestroy(h->async_graph);
  if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
  delete h;
  return GBN_OK;
}

int gbn_create(gbn_handle* out, const gbn_model_desc* md, const gbn_config* cfg) {
  if (!out || !md || !cfg) return fail(nullptr, GBN_ERR_INVALID_ARG, "gbn_create: null argument");
  *out = nullptr;
  if (cfg->num_chains <= 0) return fail(nullptr, GBN_ERR_INVALID_ARG, "num_chains must be positive");
  if (cfg->first_chain < 0 || (int64_t)cfg->first_chain + cfg->num_chains > INT32_MAX)
    return fail(nullptr, GBN_ERR_INVALID_ARG, "first_chain must be >= 0 (with first_chain + num_chains < 2^31)");
  if (cfg->algo != GBN_ALGO_NUTS && cfg->algo != GBN_ALGO_HMC)
    return fail(nullptr, GBN_ERR_INVALID_ARG, "algo must be NUTS or HMC");
  if (cfg->max_tree_depth < 1 || cfg->max_tree_depth > 20 || cfg->max_tree_depth_warmup < 1 ||
      cfg->max_tree_depth_warmup > 20)
    return fail(nullptr, GBN_ERR_INVALID_ARG, "max_tree_depth must be in [1, 20]");
  if (cfg->algo == GBN_ALGO_HMC && cfg->num_steps <= 0 && !(cfg->trajectory_length > 0))
    return fail(nullptr, GBN_ERR_INVALID_ARG, "HMC needs num_steps or trajectory_length");
  gbn_handle h = new gbn_handle_s();
  h->cfg = *cfg;
  ModelDev& m = h->m;
  m.family = md->family;
  m.num_models = md->num_models > 0 ? md->num_models : 1;
  m.n = md->n;
  m.p = md->p;
  m.precision = cfg->precision;
  for (int k = 0; k < 8; ++k) m.hyper[k] = md->hyper[k];
  int C = cfg->num_chains;
  h->C = C;
  std::vector<int32_t> chain_dim;
  cudaError_t ce = cudaSuccess;
  switch (m.family) {
    case GBN_FAMILY_HIER_NC: {
      if (!md->y || !md->sigma || !md->offsets || md->n <= 0) {
        gbn_destroy(h);
        return fail(nullptr, GBN_ERR_INVALID_ARG, "HIER_NC needs y, sigma, offsets");
      }
      int cpm = cfg->chains_per_model > 0 ? cfg->chains_per_model : C / m.num_models;
      if (cpm * m.num_models != C) {
        gbn_destroy(h);
        return fail(nullptr, GBN_ERR_SHAPE, "num_chains must equal num_models * chains_per_model");
      }
      m.chains_per_model = cpm;
      int Dmax = 0;
      for (int k = 0; k < m.num_models; ++k) {
        int J = md->offsets[k + 1] - md->offsets[k];
        if (J < 0 || md->offsets[k + 1] > md->n) {
          gbn_destroy(h);
          return fail(nullptr, GBN_ERR_SHAPE, "HIER_NC offsets out of range");
        }
        Dmax = std::max(Dmax, J + 2);
      }
      m.D = Dmax;
      chain_dim.resize(C);
      for (int c = 0; c < C; ++c) {
        int k = c / cpm;
        chain_dim[c] = md->offsets[k + 1] - md->offsets[k] + 2;
      }
      if (m.hyper[0] <= 0) m.hyper[0] = 5.0;
      if (m.hyper[1] <= 0) m.hyper[1] = 5.0;
      ce = dalloc(h, &m.y, md->n);
      if (ce == cudaSuccess) ce = dalloc(h, &m.sigma, md->n);
      if (ce == cudaSuccess) ce = dalloc(h, &m.offsets, m.num_models + 1);
      if (ce == cudaSuccess) ce = cudaMemcpy(m.y, md->y, sizeof(float) * md->n, cudaMemcpyHostToDevice);
      if (ce == cudaSuccess) ce = cudaMemcpy(m.sigma, md->sigma, sizeof(float) * md->n, cudaMemcpyHostToDevice);
      if (ce == cudaSuccess)
        ce = cudaMemcpy(m.offsets, md->offsets, sizeof(int32_t) * (m.num_models + 1), cudaMemcpyHostToDevice);
      {
        // 1/sigma per group and, per model, the constant of its potential (hier_potential.cuh)
        const double LOG_2PI = 1.8378770664093453, LOG_PI = 1.1447298858494002, LOG_2 = 0.6931471805599453;
        std::vector<float> sinv((size_t)md->n);
        std::vector<double> cmodel((size_t)m.num_models);
        for (int64_t j = 0; j < md->n; ++j) sinv[(size_t)j] = (float)(1.0 / (double)md->sigma[j]);
        for (int k = 0; k < m.num_models; ++k) {
          double c0 = 0.5 * LOG_2PI + log(m.hyper[0]) + LOG_PI + log(m.hyper[1]) - LOG_2;
          for (int j = md->offsets[k]; j < md->offsets[k + 1]; ++j) c0 += log((double)md->sigma[j]) + LOG_2PI;
          cmodel[(size_t)k] = c0;
        }
        if (ce == cudaSuccess) ce = dalloc(h, &m.hier_sinv, md->n);
        if (ce == cudaSuccess) ce = dalloc(h, &m.hier_cmodel, (size_t)m.num_models);
        if (ce == cudaSuccess)
          ce = cudaMemcpy(m.hier_sinv, sinv.data(), sizeof(float) * sinv.size(), cudaMemcpyHostToDevice);
        if (ce == cudaSuccess)
          ce = cudaMemcpy(m.hier_cmodel, cmodel.data(), sizeof(double) * cmodel.size(), cudaMemcpyHostToDevice);
      }
      break;
    }
    case GBN_FAMILY_LOGREG:
    case GBN_FAMILY_HORSESHOE: {
      if (!md->x || !md->y || md->n <= 0 || md->p <= 0) {
        gbn_destroy(h);
        return fail(nullptr, GBN_ERR_INVALID_ARG, "GLM families need x [n][p] and y [n]");
      }
      if (m.family == GBN_FAMILY_LOGREG && md->p > 64) {
        gbn_destroy(h);
        return fail(nullptr, GBN_ERR_UNSUPPORTED, "LOGREG supports p <= 64 features");
      }
      m.D = (m.family == GBN_FAMILY_LOGREG) ? md->p : 2 * md->p + 2;
      if (m.family == GBN_FAMILY_LOGREG && m.hyper[0] <= 0) m.hyper[0] = 1.0;
      size_t nx = (size_t)md->n * md->p;
      ce = dalloc(h, &m.x, nx);
      if (ce == cudaSuccess) ce = dalloc(h, &m.y, md->n);
      if (ce == cudaSuccess) ce = cudaMemcpy(m.x, md->x, sizeof(float) * nx, cudaMemcpyHostToDevice);
      if (ce == cudaSuccess) ce = cudaMemcpy(m.y, md->y, sizeof(float) * md->n, cudaMemcpyHostToDevice);
      if (ce == cudaSuccess && m.family == GBN_FAMILY_HORSESHOE) {
        // operand layouts of the horseshoe GEMMs: X^T and X, rows zero-padded to 4 floats
        const size_t n = (size_t)md->n, p = (size_t)md->p, np4 = (size_t)pad4((int)n), pp4 = (size_t)pad4((int)p);
        std::vector<float> xt(p * np4, 0.0f), xp(n * pp4, 0.0f);
        for (size_t r = 0; r < n; ++r)
          for (size_t k = 0; k < p; ++k) {
            xt[k * np4 + r] = md->x[r * p + k];
            xp[r * pp4 + k] = md->x[r * p + k];
          }
        ce = dalloc(h, &m.hs_xt, xt.size());
        if (ce == cudaSuccess) ce = dalloc(h, &m.hs_xp, xp.size());
        if (ce == cudaSuccess) ce = cudaMemcpy(m.hs_xt, xt.data(), sizeof(float) * xt.size(), cudaMemcpyHostToDevice);
        if (ce == cudaSuccess) ce = cudaMemcpy(m.hs_xp, xp.data(), sizeof(float) * xp.size(), cudaMemcpyHostToDevice);
      }
      break;
    }
    case GBN_FAMILY_SV: {
      if (!md->y || md->n <= 1) {
        gbn_destroy(h);
        return fail(nullptr, GBN_ERR_INVALID_ARG, "SV needs returns y [T], T >= 2");
      }
      m.D = (int)md->n + 2;
      if (m.hyper[0] <= 0) m.hyper[0] = 10.0;
      if (m.hyper[1] <= 0) m.hyper[1] = 0.1;
      ce = dalloc(h, &m.y, md->n);
      if (ce == cudaSuccess) ce = cudaMemcpy(m.y, md->y, sizeof(float) * md->n, cudaMemcpyHostToDevice);
      break;
    }
    default:
      gbn_destroy(h);
      return fail(nullptr, GBN_ERR_UNSUPPORTED, "unknown model family");
  }
  if (ce != cudaSuccess) {
    int r = cuda_fail(nullptr, ce, "gbn_create: model upload");
    gbn_destroy(h);
    return r;
  }
  int D = m.D;
  h->D = D;
  h->maxd = std::max(cfg->max_tree_depth, cfg->max_tree_depth_warmup);
  size_t CD = (size_t)C * D;
  EngineBufs& e = h->e;
  float** vecs[] = {&e.z_l, &e.r_l, &e.g_l, &e.z_r, &e.r_r, &e.g_r, &e.z_p,
                    &e.g_p, &e.z_sp, &e.g_sp, &e.rsum, &e.rsum_sub, &e.Q, &e.G};
  for (float** v : vecs)
    if (ce == cudaSuccess) ce = dalloc(h, v, CD);
  if (cfg->dense_mass && (m.family == GBN_FAMILY_SV || D > 1024)) {
    gbn_destroy(h);
    return fail(nullptr, GBN_ERR_UNSUPPORTED,
                "dense_mass=True needs a latent dimension <= 1024 (a warp per chain; not the SV family)");
  }
  if (cfg->mass_blocks && !cfg->dense_mass) {
    gbn_destroy(h);
    return fail(nullptr, GBN_ERR_INVALID_ARG, "mass_blocks needs dense_mass = 1");
  }
  if (cfg->mass_blocks) {
    for (int d = 0; d < D; ++d)
      if (cfg->mass_blocks[d] < -1) {
        gbn_destroy(h);
        return fail(nullptr, GBN_ERR_INVALID_ARG, "mass_blocks entries must be >= -1");
      }
    int32_t* mb = nullptr;
    if (ce == cudaSuccess) ce = dalloc(h, &mb, (size_t)D);
    if (ce == cudaSuccess) ce = cudaMemcpy(mb, cfg->mass_blocks, sizeof(int32_t) * D, cudaMemcpyHostToDevice);
    h->hp.mass_block = mb;
  }
  if (ce == cudaSuccess && cfg->dense_mass) ce = dalloc(h, &e.tmp, CD);
  if (ce == cudaSuccess && cfg->dense_mass) ce = dalloc(h, &e.tmpd, 2 * CD);
  if (ce == cudaSuccess) ce = dalloc(h, &e.r_ck, CD * h->maxd);
  if (ce == cudaSuccess) ce = dalloc(h, &e.rs_ck, CD * h->maxd);
  if (ce == cudaSuccess) ce = dalloc(h, &e.PE, (size_t)C);
  if (ce == cudaSuccess) ce = dalloc(h, &e.ctl, (size_t)C);
  if (ce == cudaSuccess && !chain_dim.empty()) {
    ce = dalloc(h, &e.chain_dim, (size_t)C);
    if (ce == cudaSuccess)
      ce = cudaMemcpy(e.chain_dim, chain_dim.data(), sizeof(int32_t) * C, cudaMemcpyHostToDevice);
  }
  // persistent engines (hierarchical and stochastic-volatility families, non-lock-step);
  // the hierarchical queue is ordered longest chain first
  h->persistent = ((m.family == GBN_FAMILY_HIER_NC || m.family == GBN_FAMILY_SV) && cfg->engine == GBN_ENGINE_FUSED);
  // the SV family always runs a CTA per chain, so its tick, plain and persistent engines share
  // one reduction order and stay bit-identical
  h->cta_per_chain = (m.family == GBN_FAMILY_SV) || D > 1024;
  if (ce == cudaSuccess && h->persistent && m.family == GBN_FAMILY_HIER_NC) {
    std::vector<int32_t> order(C);
    for (int c = 0; c < C; ++c) order[c] = c;
    if (!chain_dim.empty())
      std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return chain_dim[a] > chain_dim[b]; });
    ce = dalloc(h, &h->order, (size_t)C);
    if (ce == cudaSuccess) ce = cudaMemcpy(h->order, order.data(), sizeof(int32_t) * C, cudaMemcpyHostToDevice);
  }
  if (ce == cudaSuccess) ce = dalloc(h, &h->counters, 8);
  if (ce == cudaSuccess) ce = dalloc(h, &h->flags, (size_t)C);
  if (ce == cudaSuccess) ce = dalloc(h, &h->err_word, 4);
  if (ce == cudaSuccess) ce = dalloc(h, &h->dP, 1);
  if (ce == cudaSuccess) ce = dalloc(h, &h->vjp_pe, (size_t)C);
  h->vjp_cap = C;
  if (ce == cudaSuccess) ce = dalloc(h, &h->async_iter, 2);
  if (ce == cudaSuccess) ce = dalloc(h, &h->done_count, 2);  // one transition: gbn_sample(_async)
  h->done_cap = 2;
  if (ce == cudaSuccess) ce = cudaMallocHost((void**)&h->h_counters, sizeof(int32_t) * 8);
  if (ce == cudaSuccess) ce = cudaEventCreate(&h->ev0);
  if (ce == cudaSuccess) ce = cudaEventCreate(&h->ev1);
  if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking);
  {
    const char* g = getenv("GBN_CUDA_GRAPHS");  // "0" launches every tick directly
    h->use_graphs = !(g && g[0] == '0');
    const char* f = getenv("GBN_FUSE_TICK");  // "0": the tensor-core potentials' split and finish
    h->fuse_tick = !(f && f[0] == '0');       // run as their own kernels
  }
  if (ce == cudaSuccess && m.family == GBN_FAMILY_LOGREG && m.precision == GBN_PREC_BF16X3) {
    if (!logreg_tc_supported(m)) {
      gbn_destroy(h);
      return fail(nullptr, GBN_ERR_UNSUPPORTED, "bf16x3 tensor-core logistic path unavailable for this shape");
    }
    ce = logreg_tc_prepare(m, C);
    if (ce == cudaErrorNotSupported) {
      gbn_destroy(h);
      return fail(nullptr, GBN_ERR_UNSUPPORTED,
                  "bf16x3 needs a design matrix exactly representable in bfloat16 (use precision fp32)");
    }
  }
  if (ce == cudaSuccess && m.family == GBN_FAMILY_HORSESHOE && m.precision == GBN_PREC_BF16X3) {
    if (!horseshoe_tc_supported(m)) {
      gbn_destroy(h);
      return fail(nullptr, GBN_ERR_UNSUPPORTED, "bf16x3 tensor-core horseshoe path unavailable on this GPU");
    }
    ce = horseshoe_tc_prepare(m, C);
  }
  if (ce == cudaSuccess) ce = ensure_potential_scratch(m, C);
  if (ce == cudaSuccess && m.family == GBN_FAMILY_LOGREG && !(m.precision == GBN_PREC_BF16X3 && m.tc))
    ce = logreg_simt_smem_attr();  // before any graph capture of its launches
  if (ce != cudaSuccess) {
    int r = cuda_fail(nullptr, ce, "gbn_create: allocation");
    gbn_destroy(h);
    return r == GBN_ERR_CUDA ? GBN_ERR_OOM : r;
  }
  // launch shapes of the potential from the autotuner (GBN_AUTOTUNE=0 keeps the defaults)
  {
    const char* at = getenv("GBN_AUTOTUNE");
    if (!(at && at[0] == '0')) {
      ce = cudaMemset(e.Q, 0, sizeof(float) * CD);
      if (ce == cudaSuccess) ce = autotune_potential(m, e.Q, C, e.PE, e.G, 0, &h->tuning);
      if (ce != cudaSuccess) {
        int r = cuda_fail(nullptr, ce, "gbn_create: autotune");
        gbn_destroy(h);
        return r;
      }
    }
  }
  // static parameters
  AdvParams& P = h->hp;
  P.e = e;
  P.C = C;
  P.D = D;
  P.maxd = h->maxd;
  P.mtd_warmup = cfg->max_tree_depth_warmup;
  P.mtd = cfg->max_tree_depth;
  P.algo = cfg->algo;
  P.adapt_step = cfg->adapt_step_size;
  P.adapt_mass = cfg->adapt_mass_matrix;
  P.regularize = cfg->regularize_mass_matrix;
  P.heuristic = cfg->find_heuristic_step_size;
  P.lockstep = (cfg->engine == GBN_ENGINE_PLAIN);
  P.dense = cfg->dense_mass ? 1 : 0;
  P.fixed_steps = cfg->num_steps;
  P.target_accept = (float)cfg->target_accept_prob;
  P.max_dE = cfg->max_delta_energy > 0 ? cfg->max_delta_energy : 1000.0;
  P.traj_len = cfg->trajectory_length;
  P.seed.lo = (uint32_t)(cfg->seed & 0xffffffffu);
  P.seed.hi = (uint32_t)(cfg->seed >> 32);
  P.counters = h->counters;
  P.error_word = h->err_word;
  P.thinning = 1;
  refresh_fusion(h);
  {
    std::lock_guard<std::mutex> lock(g_handles_mu);
    h->id = g_next_id++;
    g_handles[h->id] = h;
  }
  *out = h;
  return GBN_OK;
}

int gbn_potential_and_grad(gbn_handle h, void* stream, const float* d_z, int32_t num_points, double* d_pe,
                           float* d_grad) {
  if (!h || !d_z || !d_pe || !d_grad || num_points <= 0)
    return fail(h, GBN_ERR_INVALID_ARG, "gbn_potential_and_grad: bad argument");
  cudaError_t e = launch_potential(h->m, d_z, num_points, d_pe, d_grad, nullptr, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(h, e, "potential launch");
  return GBN_OK;
}

int gbn_potential_vjp(gbn_handle h, void* stream, const float* d_z, int32_t num_points, const double* d_cot,
                      float* d_out) {
  if (!h || !d_z || !d_cot || !d_out || num_points <= 0)
    return fail(h, GBN_ERR_INVALID_ARG, "gbn_potential_vjp: bad argument");
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaSuccess;
  if (num_points > h->vjp_cap) {  // only for more points than the handle's chains
    if (h->vjp_pe) {
      cudaStreamSynchronize(st);
      cudaFree(h->vjp_pe);
      h->allocs.erase(std::find(h->allocs.begin(), h->allocs.end(), (void*)h->vjp_pe));
      h->vjp_pe = nullptr;
    }
    e = dalloc(h, &h->vjp_pe, (size_t)num_points);
    if (e != cudaSuccess) return cuda_fail(h, e, "vjp scratch");
    h->vjp_cap = num_points;
  }
  e = launch_potential(h->m, d_z, num_points, h->vjp_pe, d_out, nullptr, st);
  if (e == cudaSuccess) e = launch_scale_rows(d_cot, d_out, num_points, h->D, st);
  if (e != cudaSuccess) return cuda_fail(h, e, "vjp launch");
  return GBN_OK;
}

static cudaError_t upload_params(gbn_handle h, cudaStream_t st) {
  return cudaMemcpyAsync(h->dP, &h->hp, sizeof(AdvParams), cudaMemcpyHostToDevice, st);
}

// One batch of TICK_BATCH ticks: advance + potential, parities 0, 1, 0, ... (so every batch
// issues the same launches with the same arguments; the kernels read their parameters from
// device memory).
constexpr int TICK_BATCH = 16;
static cudaError_t launch_tick_batch(gbn_handle h, cudaStream_t st) {
  for (int k = 0; k < TICK_BATCH; ++k) {
    const int parity = k & 1;
    launch_advance(h->dP, h->C, h->D, h->cta_per_chain, h->hp.dense != 0, parity, st);
    cudaError_t e = launch_potential(h->m, h->e.Q, h->C, h->e.PE, h->e.G, h->counters + 2 * parity, st,
                                     h->hp.lrf_part_g != nullptr || h->hp.hsf_part_gb != nullptr);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Capture one batch on the private capture stream (nothing executes) and instantiate it.
// Any failure turns graphs off for this handle; the direct launches remain.
static void capture_tick_graph(gbn_handle h) {
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaError_t el = launch_tick_batch(h, h->cap_stream);
    e = cudaStreamEndCapture(h->cap_stream, &g);
    if (el != cudaSuccess) e = el;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&h->tick_graph, g, 0);
  if (g) cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    h->tick_graph = nullptr;
    h->use_graphs = 0;
    cudaGetLastError();  // capture errors are not sticky; clear the last-error slot
  } else {
    h->graph_scratch = h->m.part_g ? (void*)h->m.part_g : (void*)h->m.resid;
  }
}

// Alternate advance/potential until no chain is active.  Returns GBN status.  After the first
// batch has run directly (allocating any scratch on the way), later batches replay one CUDA
// graph of the batch.
static int tick_loop(gbn_handle h, cudaStream_t st, int64_t max_ticks) {
  int64_t ticks = 0;
  int64_t launches = 0;
  for (;;) {
    const int last = (TICK_BATCH - 1) & 1;
    void* scratch = h->m.part_g ? (void*)h->m.part_g : (void*)h->m.resid;
    if (h->tick_graph && h->graph_scratch != scratch) {  // scratch was reallocated since the capture
      cudaGraphExecDestroy(h->tick_graph);
      h->tick_graph = nullptr;
    }
    cudaError_t e;
    if (h->tick_graph) {
      e = cudaGraphLaunch(h->tick_graph, st);
    } else {
      e = launch_tick_batch(h, st);
      if (e == cudaSuccess && h->use_graphs && ticks > 0) capture_tick_graph(h);
    }
    if (e != cudaSuccess) return cuda_fail(h, e, "tick launch");
    ticks += TICK_BATCH;
    launches += TICK_BATCH;
    e = cudaMemcpyAsync(h->h_counters, h->counters, sizeof(int32_t) * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(h, e, "tick loop");
    if ((h->m.tc && logreg_tc_error(h->m)) || (h->m.hs_tc && horseshoe_tc_error(h->m)))
      return fail(h, GBN_ERR_TIMEOUT, "tensor-core potential: a device wait timed out");
    if (h->h_counters[2 * last + 1] == 0) break;
    if (ticks > max_ticks) return fail(h, GBN_ERR_TIMEOUT, "tick budget exhausted: chains did not finish");
  }
  h->stats.ticks += ticks;
  h->stats.potential_launches += launches;
  return GBN_OK;
}

int gbn_init(gbn_handle h, void* stream, int32_t num_warmup, const float* d_init_z, const float* d_inv_mass,
             gbn_state* st) {
  if (!h || !state_ok(st) || num_warmup < 0) return fail(h, GBN_ERR_INVALID_ARG, "gbn_init: bad argument");
  cudaStream_t s = (cudaStream_t)stream;
  h->num_warmup = num_warmup;
  std::vector<int> ends = adaptation_window_ends(num_warmup);
  if (ends.empty()) ends.push_back(-1);
  h->num_windows = (int)ends.size();
  if (h->window_end) {
    cudaFree(h->window_end);
    h->allocs.erase(std::find(h->allocs.begin(), h->allocs.end(), (void*)h->window_end));
    h->window_end = nullptr;
  }
  cudaError_t e = dalloc(h, &h->window_end, ends.size());
  if (e == cudaSuccess)
    e = cudaMemcpy(h->window_end, ends.data(), sizeof(int32_t) * ends.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(h, e, "gbn_init: schedule");
  AdvParams& P = h->hp;
  fill_state(P, st);
  P.window_end = h->window_end;
  P.num_windows = num_warmup > 0 ? h->num_windows : 0;
  P.num_warmup = num_warmup;
  P.col = CollectBufs{};
  P.num_collect = 0;
  P.collect_start = 0;
  P.thinning = 1;
  refresh_fusion(h);
  e = upload_params(h, s);
  if (e != cudaSuccess) return cuda_fail(h, e, "gbn_init: params");
  launch_set_rng_chain(st->rng_key, h->C, h->cfg.first_chain, s);
  int C = h->C, D = h->D;
  if (d_init_z) {
    e = cudaMemcpyAsync(st->z, d_init_z, sizeof(float) * (size_t)C * D, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess)
      e = launch_potential(h->m, st->z, C, st->potential_energy, st->z_grad, nullptr, s);
    if (e != cudaSuccess) return cuda_fail(h, e, "gbn_init: potential");
  } else {
    // find_valid_initial_params: up to 100 draws of init_to_uniform(radius=2)
    launch_init_uniform(h->dP, C, D, 0, nullptr, s);
    bool ok = false;
    for (int attempt = 0; attempt < 100; ++attempt) {
      e = launch_potential(h->m, st->z, C, st->potential_energy, st->z_grad, nullptr, s);
      if (e == cudaSuccess) e = cudaMemsetAsync(h->counters + 6, 0, sizeof(int32_t), s);
      if (e != cudaSuccess) return cuda_fail(h, e, "gbn_init: potential");
      launch_check_valid(h->dP, C, h->flags, h->counters + 6, s);
      e = cudaMemcpyAsync(h->h_counters + 6, h->counters + 6, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) return cuda_fail(h, e, "gbn_init: validity");
      if (h->h_counters[6] == 0) {
        ok = true;
        break;
      }
      launch_init_uniform(h->dP, C, D, attempt + 1, h->flags, s);
    }
    if (!ok)
      return fail(h, GBN_ERR_INIT_FAILED,
                  "Cannot find valid initial parameters. Please check your model again.");
  }
  launch_init_state(h->dP, C, D, h->hp.dense ? nullptr : d_inv_mass, (float)h->cfg.init_step_size, s);
  if (h->hp.dense) launch_init_dense_mass(h->dP, C, d_inv_mass, s);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(h, e, "gbn_init: state");
  if (h->cfg.adapt_step_size && h->cfg.find_heuristic_step_size && num_warmup > 0) {
    e = cudaMemsetAsync(h->counters, 0, sizeof(int32_t) * 4, s);
    if (e != cudaSuccess) return cuda_fail(h, e, "gbn_init: counters");
    launch_set_phase(h->dP, C, PH_HEUR_START, 0, s);
    int r = tick_loop(h, s, 1 << 20);
    if (r != GBN_OK) return r;
  }
  h->initialised = 1;
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(h, e, "gbn_init");
  return GBN_OK;
}

int gbn_run(gbn_handle h, void* stream, gbn_state* st, int32_t num_iterations, int32_t collect_start,
            int32_t thinning, gbn_collect* out) {
  if (!h || !state_ok(st) || num_iterations < 0 || thinning < 1 || collect_start < 0)
    return fail(h, GBN_ERR_INVALID_ARG, "gbn_run: bad argument");
  if (!h->window_end) return fail(h, GBN_ERR_INVALID_ARG, "gbn_run: call gbn_init first");
  if (num_iterations == 0) return GBN_OK;
  cudaStream_t s = (cudaStream_t)stream;
  AdvParams& P = h->hp;
  fill_state(P, st);
  P.col = CollectBufs{};
  if (out) {
    P.col.samples = out->samples;
    P.col.num_steps = out->num_steps;
    P.col.accept_prob = out->accept_prob;
    P.col.diverging = out->diverging;
    P.col.potential_energy = out->potential_energy;
    P.col.step_size = out->step_size;
  }
  P.collect_start = collect_start;
  P.thinning = thinning;
  P.num_collect = (collect_start < num_iterations) ? (num_iterations - collect_start + thinning - 1) / thinning : 0;
  if (!out) P.num_collect = 0;
  cudaError_t e = cudaSuccess;
  if (h->done_cap < num_iterations + 1) {
    if (h->done_count) {
      cudaFree(h->done_count);
      h->allocs.erase(std::find(h->allocs.begin(), h->allocs.end(), (void*)h->done_count));
    }
    h->done_count = nullptr;
    e = dalloc(h, &h->done_count, (size_t)num_iterations + 1);
    if (e != cudaSuccess) return cuda_fail(h, e, "gbn_run: barrier counts");
    h->done_cap = num_iterations + 1;
  }
  P.done_count = h->done_count;
  refresh_fusion(h);
  e = upload_params(h, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(h->done_count, 0, sizeof(int32_t) * (num_iterations + 1), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(h->counters, 0, sizeof(int32_t) * 4, s);
  if (e != cudaSuccess) return cuda_fail(h, e, "gbn_run: setup");
  launch_set_phase(h->dP, h->C, PH_START, num_iterations, s);
  int64_t per_iter = (h->cfg.algo == GBN_ALGO_HMC) ? 4096 : ((int64_t)1 << h->maxd) + 8;
  if (h->cfg.find_heuristic_step_size) per_iter += 512;
  int64_t max_ticks = (int64_t)num_iterations * per_iter * (P.lockstep ? 2 : 1) + 4096;
  cudaEventRecord(h->ev0, s);
  int r = GBN_OK;
  if (h->persistent) {
    // one launch: every chain runs all its transitions from the device work queue
    e = cudaMemsetAsync(h->counters + 7, 0, sizeof(int32_t), s);
    if (e != cudaSuccess) return cuda_fail(h, e, "gbn_run: queue");
    if (h->m.family == GBN_FAMILY_SV) {
      SvView sv{h->m.y, (int)h->m.n, h->m.hyper[2] != 0.0, h->m.hyper[0], h->m.hyper[1]};
      launch_persistent_sv(h->dP, sv, h->counters + 7, h->C, h->D, s);
    } else {
      HierView hv{h->m.y, h->m.hier_sinv, h->m.hier_cmodel, h->m.offsets, h->m.chains_per_model, h->m.num_models,
                  (float)(1.0 / (h->m.hyper[0] * h->m.hyper[0])), (float)(1.0 / h->m.hyper[1])};
      launch_persistent_hier(h->dP, hv, h->counters + 7, h->order, h->C, h->hp.dense != 0, s);
    }
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(h, e, "gbn_run: persistent engine");
  } else {
    r = tick_loop(h, s, max_ticks);
  }
  cudaEventRecord(h->ev1, s);
  if (r != GBN_OK) return r;
  cudaEventSynchronize(h->ev1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  h->stats.device_ms = ms;
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(h, e, "gbn_run");
  return GBN_OK;
}

int gbn_sample(gbn_handle h, void* stream, gbn_state* st) { return gbn_run(h, stream, st, 1, 0, 1, nullptr); }

// Builds the graph of gbn_sample_async's tick loop: a WHILE node whose body is one batch of
// ticks followed by the condition kernel.  Every kernel reads its parameters from device memory
// (the AdvParams block, the counters), so one graph serves every later call of the handle.
static cudaError_t build_async_graph(gbn_handle h) {
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaGraphCreate(&g, 0);
  cudaGraphConditionalHandle ch = 0;
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&ch, g, 1, cudaGraphCondAssignDefault);
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = ch;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node = nullptr;
  if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
  if (e == cudaSuccess) {
    cudaGraph_t body = np.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(h->cap_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      cudaError_t el = launch_tick_batch(h, h->cap_stream);
      const int* tc_err = h->m.tc ? logreg_tc_error_ptr(h->m) : (h->m.hs_tc ? horseshoe_tc_error_ptr(h->m) : nullptr);
      launch_tick_condition((unsigned long long)ch, h->counters, (TICK_BATCH - 1) & 1, h->async_iter, tc_err,
                            h->err_word, h->cap_stream);
      e = cudaStreamEndCapture(h->cap_stream, &body);
      if (el != cudaSuccess) e = el;
    }
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&h->async_graph, g, 0);
  if (g) cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    h->async_graph = nullptr;
    cudaGetLastError();
  }
  return e;
}

int gbn_sample_async(gbn_handle h, void* stream, gbn_state* st) {
  if (!h || !state_ok(st)) return fail(h, GBN_ERR_INVALID_ARG, "gbn_sample_async: bad argument");
  if (!h->window_end) return fail(h, GBN_ERR_INVALID_ARG, "gbn_sample_async: call gbn_init first");
  cudaStream_t s = (cudaStream_t)stream;
  AdvParams& P = h->hp;
  fill_state(P, st);
  P.col = CollectBufs{};
  P.collect_start = 0;
  P.thinning = 1;
  P.num_collect = 0;
  P.done_count = h->done_count;  // sized for one transition at gbn_create
  refresh_fusion(h);
  cudaError_t e = cudaSuccess;
  void* scratch = h->m.part_g ? (void*)h->m.part_g : (void*)h->m.resid;
  if (h->async_graph && h->async_scratch != scratch) {  // scratch was reallocated since the build
    cudaGraphExecDestroy(h->async_graph);
    h->async_graph = nullptr;
  }
  if (!h->persistent && !h->async_graph) {  // first call of the handle: build the tick-loop graph
    int64_t per_iter = (h->cfg.algo == GBN_ALGO_HMC) ? 4096 : ((int64_t)1 << h->maxd) + 8;
    if (h->cfg.find_heuristic_step_size) per_iter += 512;
    const int64_t max_ticks = per_iter * (P.lockstep ? 2 : 1) + 4096;
    const int32_t budget[2] = {0, (int32_t)(max_ticks / TICK_BATCH + 1)};
    e = cudaMemcpy(h->async_iter, budget, sizeof(budget), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = build_async_graph(h);
    if (e != cudaSuccess) return cuda_fail(h, e, "gbn_sample_async: graph set-up");
    h->async_scratch = scratch;
  }
  launch_set_params(P, h->dP, s);
  e = cudaMemsetAsync(h->done_count, 0, sizeof(int32_t) * 2, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(h->counters, 0, sizeof(int32_t) * 8, s);
  if (e != cudaSuccess) return cuda_fail(h, e, "gbn_sample_async: setup");
  launch_set_phase(h->dP, h->C, PH_START, 1, s);
  if (h->persistent) {
    if (h->m.family == GBN_FAMILY_SV) {
      SvView sv{h->m.y, (int)h->m.n, h->m.hyper[2] != 0.0, h->m.hyper[0], h->m.hyper[1]};
      launch_persistent_sv(h->dP, sv, h->counters + 7, h->C, h->D, s);
    } else {
      HierView hv{h->m.y, h->m.hier_sinv, h->m.hier_cmodel, h->m.offsets, h->m.chains_per_model, h->m.num_models,
                  (float)(1.0 / (h->m.hyper[0] * h->m.hyper[0])), (float)(1.0 / h->m.hyper[1])};
      launch_persistent_hier(h->dP, hv, h->counters + 7, h->order, h->C, h->hp.dense != 0, s);
    }
  } else {
    e = cudaMemsetAsync(h->async_iter, 0, sizeof(int32_t), s);
    if (e == cudaSuccess) e = cudaGraphLaunch(h->async_graph, s);
    if (e != cudaSuccess) return cuda_fail(h, e, "gbn_sample_async: launch");
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(h, e, "gbn_sample_async");
  return GBN_OK;
}

int gbn_check_async(gbn_handle h, void* stream) {
  if (!h) return fail(h, GBN_ERR_INVALID_ARG, "gbn_check_async: null handle");
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(h, e, "gbn_check_async");
  int32_t w = 0;
  e = cudaMemcpy(&w, h->err_word, sizeof(int32_t), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(h, e, "gbn_check_async");
  if (w != 0) {
    cudaMemset(h->err_word, 0, sizeof(int32_t));
    return fail(h, GBN_ERR_TIMEOUT, "an asynchronous transition exhausted its tick budget or a device wait timed out");
  }
  if ((h->m.tc && logreg_tc_error(h->m)) || (h->m.hs_tc && horseshoe_tc_error(h->m)))
    return fail(h, GBN_ERR_TIMEOUT, "tensor-core potential: a device wait timed out");
  return GBN_OK;
}

const char* gbn_tuning(gbn_handle h) { return h ? h->tuning.c_str() : ""; }

int gbn_time_potential(gbn_handle h, void* stream, int32_t reps, float* ms) {
  if (!h || !ms || reps < 1) return fail(h, GBN_ERR_INVALID_ARG, "gbn_time_potential: bad argument");
  cudaStream_t s = (cudaStream_t)stream;
  refresh_fusion(h);
  const bool fused = h->hp.lrf_part_g != nullptr || h->hp.hsf_part_gb != nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  // the chains' last query positions; the engine's G and PE are rewritten before they are read again
  if (e == cudaSuccess) e = launch_potential(h->m, h->e.Q, h->C, h->e.PE, h->e.G, nullptr, s, fused);
  if (e == cudaSuccess) e = cudaEventRecord(a, s);
  for (int r = 0; r < reps && e == cudaSuccess; ++r)
    e = launch_potential(h->m, h->e.Q, h->C, h->e.PE, h->e.G, nullptr, s, fused);
  if (e == cudaSuccess) e = cudaEventRecord(b, s);
  if (e == cudaSuccess) e = cudaEventSynchronize(b);
  float t = 0.0f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, a, b);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (e != cudaSuccess) return cuda_fail(h, e, "gbn_time_potential");
  *ms = t / (float)reps;
  return GBN_OK;
}

int gbn_measure_sfu(void* stream, int32_t mode, double* ops_per_second) {
  if (!ops_per_second || mode < 0 || mode > 2)
    return fail(nullptr, GBN_ERR_INVALID_ARG, "gbn_measure_sfu: bad argument");
  cudaError_t e = measure_sfu_rate(mode, (cudaStream_t)stream, ops_per_second);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "gbn_measure_sfu");
  return GBN_OK;
}

int gbn_logreg_terms(gbn_handle h, int32_t* three_term_blocks, int32_t* blocks, float* two_term_limit) {
  if (!h || !three_term_blocks || !blocks || !two_term_limit)
    return fail(h, GBN_ERR_INVALID_ARG, "gbn_logreg_terms: null argument");
  *three_term_blocks = 0;
  *blocks = 0;
  *two_term_limit = -1.0f;
  if (h->m.family != GBN_FAMILY_LOGREG || !h->m.tc) return GBN_OK;
  cudaError_t e = cudaDeviceSynchronize();
  int three = 0, nb = 0;
  if (e == cudaSuccess) e = logreg_tc_terms(h->m, &three, &nb, two_term_limit);
  if (e != cudaSuccess) return cuda_fail(h, e, "gbn_logreg_terms");
  *three_term_blocks = three;
  *blocks = nb;
  return GBN_OK;
}

int gbn_get_stats(gbn_handle h, gbn_stats* stats) {
  if (!h || !stats) return fail(h, GBN_ERR_INVALID_ARG, "gbn_get_stats: null argument");
  *stats = h->stats;
  return GBN_OK;
}

}  // extern "C"
