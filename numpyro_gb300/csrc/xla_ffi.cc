// xla_ffi.cc -- XLA FFI handlers over the C ABI, for jax.ffi (libgbnuts_xla.so).
//
// numpyro runs MCMCKernel.sample inside jit (numpyro/infer/mcmc.py:188-190, fori_collect
// numpyro/util.py:386-403) and differentiates potential_fn with value_and_grad
// (numpyro/infer/hmc_util.py:242-252).  Under jit these become custom calls: XLA owns every
// buffer, passes its CUDA stream, and may invoke a handler from any thread.  The handlers below
// therefore take the library handle as an integer attribute (gbn_handle_from_id, a
// mutex-protected registry), write only into XLA's result buffers, allocate nothing and never
// block the host:
//   gbn_xla_potential_and_grad   z [K, D] f32 -> (U [K] f64, dU/dz [K, D] f32)
//   gbn_xla_potential_vjp        z [K, D] f32, cotangent [K] f64 -> cot * dU/dz [K, D] f32
//   gbn_xla_sample               the 19 HMCState / HMCAdaptState buffers, aliased input to
//                                output (jax.ffi.ffi_call input_output_aliases), one transition
//                                by gbn_sample_async
// This file compiles only where the XLA FFI headers are available (jax.ffi.include_dir());
// numpyro_gb300/build.py builds it into libgbnuts_xla.so next to libgbnuts.so when they are.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/gbnuts.h"
#include "xla/ffi/api/ffi.h"

namespace ffi = xla::ffi;

namespace {

ffi::Error status_error(gbn_handle h, int rc) {
  if (rc == GBN_OK) return ffi::Error::Success();
  return ffi::Error(rc == GBN_ERR_INVALID_ARG ? ffi::ErrorCode::kInvalidArgument : ffi::ErrorCode::kInternal,
                    gbn_last_error(h));
}

ffi::Error PotentialAndGrad(cudaStream_t stream, int64_t handle, ffi::Buffer<ffi::F32> z,
                            ffi::ResultBuffer<ffi::F64> pe, ffi::ResultBuffer<ffi::F32> grad) {
  gbn_handle h = gbn_handle_from_id(handle);
  if (!h) return ffi::Error(ffi::ErrorCode::kInvalidArgument, "gbn_xla_potential_and_grad: unknown handle");
  const auto dims = z.dimensions();
  const int32_t k = dims.size() == 2 ? (int32_t)dims[0] : 1;
  return status_error(h, gbn_potential_and_grad(h, stream, z.typed_data(), k, pe->typed_data(),
                                                grad->typed_data()));
}

ffi::Error PotentialVjp(cudaStream_t stream, int64_t handle, ffi::Buffer<ffi::F32> z, ffi::Buffer<ffi::F64> cot,
                        ffi::ResultBuffer<ffi::F32> out) {
  gbn_handle h = gbn_handle_from_id(handle);
  if (!h) return ffi::Error(ffi::ErrorCode::kInvalidArgument, "gbn_xla_potential_vjp: unknown handle");
  const auto dims = z.dimensions();
  const int32_t k = dims.size() == 2 ? (int32_t)dims[0] : 1;
  return status_error(h, gbn_potential_vjp(h, stream, z.typed_data(), k, cot.typed_data(), out->typed_data()));
}

// Result order follows gbn_state (include/gbnuts.h); the results alias the arguments.
ffi::Error Sample(cudaStream_t stream, int64_t handle, ffi::RemainingArgs, ffi::ResultBuffer<ffi::S32> i,
                  ffi::ResultBuffer<ffi::F32> z, ffi::ResultBuffer<ffi::F32> z_grad,
                  ffi::ResultBuffer<ffi::F64> potential_energy, ffi::ResultBuffer<ffi::F64> energy,
                  ffi::ResultBuffer<ffi::S32> num_steps, ffi::ResultBuffer<ffi::F32> accept_prob,
                  ffi::ResultBuffer<ffi::F32> mean_accept_prob, ffi::ResultBuffer<ffi::U8> diverging,
                  ffi::ResultBuffer<ffi::F32> step_size, ffi::ResultBuffer<ffi::F32> inverse_mass_matrix,
                  ffi::ResultBuffer<ffi::F32> mass_matrix_sqrt, ffi::ResultBuffer<ffi::F32> mass_matrix_sqrt_inv,
                  ffi::ResultBuffer<ffi::F64> ss_state, ffi::ResultBuffer<ffi::F64> mm_mean,
                  ffi::ResultBuffer<ffi::F64> mm_m2, ffi::ResultBuffer<ffi::S32> mm_n,
                  ffi::ResultBuffer<ffi::S32> window_idx, ffi::ResultBuffer<ffi::U32> rng_key) {
  gbn_handle h = gbn_handle_from_id(handle);
  if (!h) return ffi::Error(ffi::ErrorCode::kInvalidArgument, "gbn_xla_sample: unknown handle");
  gbn_state st;
  st.i = i->typed_data();
  st.z = z->typed_data();
  st.z_grad = z_grad->typed_data();
  st.potential_energy = potential_energy->typed_data();
  st.energy = energy->typed_data();
  st.num_steps = num_steps->typed_data();
  st.accept_prob = accept_prob->typed_data();
  st.mean_accept_prob = mean_accept_prob->typed_data();
  st.diverging = diverging->typed_data();
  st.step_size = step_size->typed_data();
  st.inverse_mass_matrix = inverse_mass_matrix->typed_data();
  st.mass_matrix_sqrt = mass_matrix_sqrt->typed_data();
  st.mass_matrix_sqrt_inv = mass_matrix_sqrt_inv->typed_data();
  st.ss_state = ss_state->typed_data();
  st.mm_mean = mm_mean->typed_data();
  st.mm_m2 = mm_m2->typed_data();
  st.mm_n = mm_n->typed_data();
  st.window_idx = window_idx->typed_data();
  st.rng_key = rng_key->typed_data();
  return status_error(h, gbn_sample_async(h, stream, &st));
}

}  // namespace

XLA_FFI_DEFINE_HANDLER_SYMBOL(gbn_xla_potential_and_grad, PotentialAndGrad,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Attr<int64_t>("handle")
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F32>>());

XLA_FFI_DEFINE_HANDLER_SYMBOL(gbn_xla_potential_vjp, PotentialVjp,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Attr<int64_t>("handle")
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F32>>());

XLA_FFI_DEFINE_HANDLER_SYMBOL(gbn_xla_sample, Sample,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Attr<int64_t>("handle")
                                  .RemainingArgs()
                                  .Ret<ffi::Buffer<ffi::S32>>()   // i
                                  .Ret<ffi::Buffer<ffi::F32>>()   // z
                                  .Ret<ffi::Buffer<ffi::F32>>()   // z_grad
                                  .Ret<ffi::Buffer<ffi::F64>>()   // potential_energy
                                  .Ret<ffi::Buffer<ffi::F64>>()   // energy
                                  .Ret<ffi::Buffer<ffi::S32>>()   // num_steps
                                  .Ret<ffi::Buffer<ffi::F32>>()   // accept_prob
                                  .Ret<ffi::Buffer<ffi::F32>>()   // mean_accept_prob
                                  .Ret<ffi::Buffer<ffi::U8>>()    // diverging
                                  .Ret<ffi::Buffer<ffi::F32>>()   // step_size
                                  .Ret<ffi::Buffer<ffi::F32>>()   // inverse_mass_matrix
                                  .Ret<ffi::Buffer<ffi::F32>>()   // mass_matrix_sqrt
                                  .Ret<ffi::Buffer<ffi::F32>>()   // mass_matrix_sqrt_inv
                                  .Ret<ffi::Buffer<ffi::F64>>()   // ss_state
                                  .Ret<ffi::Buffer<ffi::F64>>()   // mm_mean
                                  .Ret<ffi::Buffer<ffi::F64>>()   // mm_m2
                                  .Ret<ffi::Buffer<ffi::S32>>()   // mm_n
                                  .Ret<ffi::Buffer<ffi::S32>>()   // window_idx
                                  .Ret<ffi::Buffer<ffi::U32>>());  // rng_key
