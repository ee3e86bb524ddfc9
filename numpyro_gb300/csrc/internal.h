// internal.h -- host-side declarations shared by the translation units of libgbnuts.
#pragma once
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

namespace gbn {

struct AdvParams;

// Launch shapes of the potential kernels, chosen by autotune_potential (defaults before tuning).
// hier_cpb: chains (warps) per CTA of the hierarchical kernel; hs_tm: rows per thread of the horseshoe
// residual GEMM (tile height 16 * hs_tm); hs_splits: row ranges of the horseshoe adjoint GEMM;
// lr_rg: row groups of the FP32 logistic kernel (0: the allocation default).
struct TuneParams {
  int hier_cpb = 8;
  int hs_tm = 4;
  int hs_splits = 4;
  int lr_rg = 0;
};

// Device copy of a registry model plus the scratch its potential needs.
struct ModelDev {
  int family = 0;
  int num_models = 1;
  int64_t n = 0;
  int p = 0;
  int D = 0;               // latent dimension (max over models)
  int chains_per_model = 1;
  float* x = nullptr;      // [n][p]
  float* y = nullptr;      // [n]
  float* sigma = nullptr;  // [n]
  int32_t* offsets = nullptr;
  double hyper[8] = {0};
  int precision = 0;
  // scratch (sized for scratch_points potential points)
  TuneParams tune;
  int scratch_points = 0;
  int row_groups = 0;       // default row groups of the FP32 logistic kernel
  int row_groups_cap = 0;   // row groups the logistic partial buffers hold
  float* part_g = nullptr;    // [row_groups][points][64]
  double* part_ll = nullptr;  // [row_groups][points]
  float* resid = nullptr;     // horseshoe [n][points]
  float* part_gb = nullptr;   // horseshoe split-K partials
  double* part_rr = nullptr;  // horseshoe [row tiles][points]
  void* tc = nullptr;         // tensor-core path state (logreg_tc.cu)
  // horseshoe: X^T [P][pad4(n)] and X [n][pad4(P)] zero-padded, beta^T scratch [pad4(P)][pad4(points)]
  float* hier_sinv = nullptr;     // hierarchical family: 1/sigma per group
  double* hier_cmodel = nullptr;  // hierarchical family: per-model constant of the potential
  float* hs_xt = nullptr;
  float* hs_xp = nullptr;
  float* hs_bt = nullptr;
  void* hs_tc = nullptr;  // horseshoe tensor-core path state (horseshoe_tc.cu)
};

// device view of the hierarchical family's data (persistent engine)
struct HierView {
  const float* y;
  const float* sinv;
  const double* cmodel;
  const int32_t* off;
  int cpm;
  int num_models;
  float inv_ms2, inv_ts;
};

// device view of the stochastic-volatility data (persistent engine)
struct SvView {
  const float* ret;
  int T;
  int noncentred;
  double s_rate, nu_rate;
};

inline int pad4(int v) { return (v + 3) & ~3; }

// nuts_engine.cu
// a CTA per chain when cta_per_chain or D > 1024, else a warp per chain
void launch_advance(const AdvParams* dP, int C, int D, bool cta_per_chain, bool dense, int parity, cudaStream_t st);
void launch_persistent_hier(const AdvParams* dP, const HierView& hv, int32_t* queue_head, const int32_t* order,
                            int C, bool dense, cudaStream_t st);
void launch_persistent_sv(const AdvParams* dP, const SvView& sv, int32_t* queue_head, int C, int D,
                          cudaStream_t st);
void launch_init_uniform(const AdvParams* dP, int C, int D, int attempt, const int32_t* flag, cudaStream_t st);
void launch_check_valid(const AdvParams* dP, int C, int32_t* flag, int32_t* count, cudaStream_t st);
void launch_init_state(const AdvParams* dP, int C, int D, const float* inv_mass_init, float init_step,
                       cudaStream_t st);
void launch_init_dense_mass(const AdvParams* dP, int C, const float* inv_mass_init, cudaStream_t st);
void launch_set_phase(const AdvParams* dP, int C, int phase, int iters, cudaStream_t st);
void launch_set_rng_chain(uint32_t* rng_key, int C, int first_chain, cudaStream_t st);
// copies a parameter block (passed by value) into device memory, in stream order
void launch_set_params(const AdvParams& p, AdvParams* dst, cudaStream_t st);
// Last node of the device-side tick loop (a CUDA-graph WHILE node): counts the iteration in
// iter[0] and keeps the loop going while a chain is active (counters[2 last + 1]), the budget
// iter[1] is not exhausted and no tensor-core wait timed out; an active chain at the budget or a
// timed-out wait sets *err_word to GBN_ERR_TIMEOUT.
void launch_tick_condition(unsigned long long cond_handle, const int32_t* counters, int last, int32_t* iter,
                           const int* tc_err, int32_t* err_word, cudaStream_t st);
cudaError_t logreg_simt_smem_attr();
// special-function unit throughput (operations/s) for mode 0 ex2, 1 tanh, 2 the logistic epilogue's mix
cudaError_t measure_sfu_rate(int mode, cudaStream_t st, double* ops_per_s);

// potentials_simt.cu: returns cudaError of the launch
cudaError_t ensure_potential_scratch(ModelDev& m, int points);
void free_potential_scratch(ModelDev& m);
// fused_tick: the tick engine's call, whose advance kernel fuses the tensor-core logistic and
// horseshoe potentials' coefficient split and finish (logreg_tc_fusion, horseshoe_tc_fusion);
// other potentials ignore it
cudaError_t launch_potential(ModelDev& m, const float* Q, int npts, double* PE, float* G,
                             const int32_t* pending, cudaStream_t st, bool fused_tick = false);
// Times the candidate launch shapes of this model's potential at npts points (Q: any valid
// [npts][D] positions; PE/G outputs) and stores the fastest in m.tune.  Decisions are cached per
// process for each (device, family, shape, points), so every handle of a shape runs the same
// arithmetic.  report receives "name=value ..." of the choice.
cudaError_t autotune_potential(ModelDev& m, const float* Q, int npts, double* PE, float* G, cudaStream_t st,
                               std::string* report);
// VJP: out[k] = cot[k] * grad U(z_k)
cudaError_t launch_scale_rows(const double* cot, float* G, int npts, int D, cudaStream_t st);

// horseshoe_tc.cu (tensor-core bf16x3 GEMMs of the horseshoe potential)
bool horseshoe_tc_supported(const ModelDev& m);
cudaError_t horseshoe_tc_prepare(ModelDev& m, int points);
void horseshoe_tc_free(ModelDev& m);
int horseshoe_tc_error(const ModelDev& m);  // nonzero: a device wait timed out
int* horseshoe_tc_error_ptr(const ModelDev& m);  // device address of that error word (or null)
cudaError_t horseshoe_tc_launch(ModelDev& m, const float* Q, int npts, double* PE, float* G, const int32_t* pending,
                                cudaStream_t st,
                                bool fused_tick = false);

// logreg_tc.cu (tensor-core BF16 split-precision logistic potential)
bool logreg_tc_supported(const ModelDev& m);
cudaError_t logreg_tc_prepare(ModelDev& m, int points);
void logreg_tc_free(ModelDev& m);
int logreg_tc_error(const ModelDev& m);  // nonzero: a device wait timed out
// blocks of the last launch that took three coefficient terms, of how many; the two-term limit
cudaError_t logreg_tc_terms(const ModelDev& m, int* three, int* blocks, float* limit);
int* logreg_tc_error_ptr(const ModelDev& m);  // device address of that error word (or null)
cudaError_t logreg_tc_launch(ModelDev& m, const float* Q, int npts, double* PE, float* G, const int32_t* pending,
                             cudaStream_t st, bool fused_tick = false);
// Fills P's lrf_* fields so the tick engine's advance kernel fuses this potential's coefficient split
// and row-group finish (launches over npts points); false when the tensor-core path is not set up.
bool logreg_tc_fusion(const ModelDev& m, int npts, AdvParams* P);
// the tensor-core horseshoe potential's coefficient split and finish fused into the tick engine
// (for the CTA-per-chain state machine only)
bool horseshoe_tc_fusion(ModelDev& m, int npts, AdvParams* P);

}  // namespace gbn
