// fire_xla.cc -- XLA FFI handlers over libfire.so: the local-energy, Metropolis-block and parameter-gradient custom
// calls that replace the reference's jitted per-walker calls (batched_energy_fn, update.py:95-100, 153-157; MCStep,
// mcmc.py:329-344; jac_fn = batched_vmap(jax.grad(log_p)), preconditioner.py:190-191) with one call over the whole
// walker batch.  Compiled only where jaxlib ships the FFI header
// (jax.ffi.include_dir()), and linked with libfire.so.
//
// Every buffer comes from XLA; the library's workspace is taken from XLA's scratch allocator, so no cudaMalloc runs
// inside a jitted step.  The status words are an output: a set flag (capacity overflow) means the caller grows the
// capacities from status[1..4] and repeats the step, as the reference's StaticScheduler does
// (static_args.py:62-84).
#include <cuda_runtime.h>

#include <cstdint>

#include "fire.h"
#include "xla/ffi/api/ffi.h"

namespace ffi = xla::ffi;

namespace {

fire_problem make_problem(int64_t n_walkers, int64_t n_el, int64_t n_nuc, int32_t n_up, float cutoff,
                          float cutoff_1el, int32_t cap_pairs, int32_t cap_nuc, int32_t precision, int32_t chunk) {
  fire_problem p{};  // refine_cap 0: no refinement pass (the handler has no host loop that sizes its capacity)
  p.n_el = static_cast<int32_t>(n_el);
  p.n_up = n_up;
  p.n_nuc = static_cast<int32_t>(n_nuc);
  p.n_walkers = static_cast<int32_t>(n_walkers);
  p.cutoff = cutoff;
  p.cutoff_1el = cutoff_1el;
  p.cap_pairs = cap_pairs;
  p.cap_nuc = cap_nuc;
  p.precision = precision;
  p.chunk_walkers = chunk;
  return p;
}

ffi::Error to_error(fire_status st, const char* what) {
  if (st == FIRE_OK) return ffi::Error::Success();
  return ffi::Error(st == FIRE_ERR_CUDA ? ffi::ErrorCode::kInternal : ffi::ErrorCode::kInvalidArgument, what);
}

// electrons [B, n_el, 3] float32; R [n_nuc, 3], Z [n_nuc] float32; prepared: fire_prepare_params's buffer.
ffi::Error LocalEnergy(cudaStream_t stream, ffi::ScratchAllocator scratch, ffi::Buffer<ffi::F32> R,
                       ffi::Buffer<ffi::F32> Z, ffi::Buffer<ffi::U8> prepared, ffi::Buffer<ffi::F32> r, int32_t n_up,
                       float cutoff, float cutoff_1el, int32_t cap_pairs, int32_t cap_nuc, int32_t precision,
                       int32_t chunk, ffi::ResultBuffer<ffi::F32> logpsi, ffi::ResultBuffer<ffi::F32> sign,
                       ffi::ResultBuffer<ffi::F32> e_loc, ffi::ResultBuffer<ffi::F64> e_stats,
                       ffi::ResultBuffer<ffi::S32> status) {
  const auto d = r.dimensions();
  if (d.size() != 3 || d[2] != 3 || precision == FIRE_PREC_FP64)
    return ffi::Error(ffi::ErrorCode::kInvalidArgument, "fire_local_energy: electrons must be float32 [B, n_el, 3]");
  fire_problem p = make_problem(d[0], d[1], R.dimensions()[0], n_up, cutoff, cutoff_1el, cap_pairs, cap_nuc,
                                precision, chunk);
  size_t bytes = 0;
  fire_status st = fire_workspace_size(&p, chunk, &bytes);
  if (st != FIRE_OK) return to_error(st, "fire_workspace_size");
  auto ws = scratch.Allocate(bytes, 256);
  if (!ws.has_value()) return ffi::Error(ffi::ErrorCode::kResourceExhausted, "fire_local_energy: workspace");
  cudaMemsetAsync(status->typed_data(), 0, FIRE_STATUS_WORDS * sizeof(int32_t), stream);
  st = fire_local_energy(stream, &p, R.typed_data(), Z.typed_data(), prepared.typed_data(), r.typed_data(),
                         logpsi->typed_data(), sign->typed_data(), e_loc->typed_data(), e_stats->typed_data(), nullptr,
                         *ws, bytes, status->typed_data());
  return to_error(st, "fire_local_energy");
}

// r_in [B, n_el, 3], logpsi_in [B] float32 (log|psi(r_in)|) -> r_out, logpsi_out after `steps` all-electron moves,
// n_accept [B] int32.  The outputs are copies of the inputs updated in place by fire_mcmc_block.
ffi::Error McmcBlock(cudaStream_t stream, ffi::ScratchAllocator scratch, ffi::Buffer<ffi::F32> R,
                     ffi::Buffer<ffi::F32> Z, ffi::Buffer<ffi::U8> prepared, ffi::Buffer<ffi::F32> r_in,
                     ffi::Buffer<ffi::F32> logpsi_in, int32_t n_up, float cutoff, float cutoff_1el, int32_t cap_pairs,
                     int32_t cap_nuc, int32_t precision, int32_t chunk, int32_t steps, float width, int64_t seed,
                     int64_t counter, ffi::ResultBuffer<ffi::F32> r_out, ffi::ResultBuffer<ffi::F32> logpsi_out,
                     ffi::ResultBuffer<ffi::S32> n_accept, ffi::ResultBuffer<ffi::S32> static_max,
                     ffi::ResultBuffer<ffi::S32> status) {
  const auto d = r_in.dimensions();
  if (d.size() != 3 || d[2] != 3 || precision == FIRE_PREC_FP64)
    return ffi::Error(ffi::ErrorCode::kInvalidArgument, "fire_mcmc_block: electrons must be float32 [B, n_el, 3]");
  fire_problem p = make_problem(d[0], d[1], R.dimensions()[0], n_up, cutoff, cutoff_1el, cap_pairs, cap_nuc,
                                precision, chunk);
  size_t bytes = 0;
  fire_status st = fire_workspace_size(&p, chunk, &bytes);
  if (st != FIRE_OK) return to_error(st, "fire_workspace_size");
  auto ws = scratch.Allocate(bytes, 256);
  if (!ws.has_value()) return ffi::Error(ffi::ErrorCode::kResourceExhausted, "fire_mcmc_block: workspace");
  cudaMemcpyAsync(r_out->typed_data(), r_in.typed_data(), r_in.size_bytes(), cudaMemcpyDeviceToDevice, stream);
  cudaMemcpyAsync(logpsi_out->typed_data(), logpsi_in.typed_data(), logpsi_in.size_bytes(), cudaMemcpyDeviceToDevice,
                  stream);
  cudaMemsetAsync(n_accept->typed_data(), 0, n_accept->size_bytes(), stream);
  cudaMemsetAsync(static_max->typed_data(), 0, static_max->size_bytes(), stream);
  cudaMemsetAsync(status->typed_data(), 0, FIRE_STATUS_WORDS * sizeof(int32_t), stream);
  st = fire_mcmc_block(stream, &p, R.typed_data(), Z.typed_data(), prepared.typed_data(), r_out->typed_data(),
                       logpsi_out->typed_data(), steps, width, static_cast<uint64_t>(seed),
                       static_cast<uint64_t>(counter), nullptr, nullptr, n_accept->typed_data(),
                       static_max->typed_data(), *ws, bytes, status->typed_data());
  return to_error(st, "fire_mcmc_block");
}

// electrons [B, n_el, 3] float32 -> grad [B, L] (d log|psi| / d parameter, the blob layout of fire_param_layout),
// logpsi [B], sign [B]: the rows of SPRING's Jacobian.
ffi::Error LogpsiGrad(cudaStream_t stream, ffi::ScratchAllocator scratch, ffi::Buffer<ffi::F32> R,
                      ffi::Buffer<ffi::U8> prepared, ffi::Buffer<ffi::F32> r, int32_t n_up, float cutoff,
                      float cutoff_1el, int32_t cap_pairs, int32_t cap_nuc, int32_t chunk,
                      ffi::ResultBuffer<ffi::F32> grad, ffi::ResultBuffer<ffi::F32> logpsi,
                      ffi::ResultBuffer<ffi::F32> sign, ffi::ResultBuffer<ffi::S32> status) {
  const auto d = r.dimensions();
  if (d.size() != 3 || d[2] != 3)
    return ffi::Error(ffi::ErrorCode::kInvalidArgument, "fire_logpsi_grad: electrons must be float32 [B, n_el, 3]");
  fire_problem p = make_problem(d[0], d[1], R.dimensions()[0], n_up, cutoff, cutoff_1el, cap_pairs, cap_nuc,
                                FIRE_PREC_FP32, chunk);
  size_t bytes = 0;
  fire_status st = fire_logpsi_grad_workspace_size(&p, chunk, &bytes);
  if (st != FIRE_OK) return to_error(st, "fire_logpsi_grad_workspace_size");
  auto ws = scratch.Allocate(bytes, 256);
  if (!ws.has_value()) return ffi::Error(ffi::ErrorCode::kResourceExhausted, "fire_logpsi_grad: workspace");
  cudaMemsetAsync(status->typed_data(), 0, FIRE_STATUS_WORDS * sizeof(int32_t), stream);
  st = fire_logpsi_grad(stream, &p, R.typed_data(), prepared.typed_data(), r.typed_data(), sign->typed_data(),
                        logpsi->typed_data(), grad->typed_data(), *ws, bytes, status->typed_data());
  return to_error(st, "fire_logpsi_grad");
}

}  // namespace

XLA_FFI_DEFINE_HANDLER_SYMBOL(FireLocalEnergy, LocalEnergy,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Ctx<ffi::ScratchAllocator>()
                                  .Arg<ffi::Buffer<ffi::F32>>()  // R
                                  .Arg<ffi::Buffer<ffi::F32>>()  // Z
                                  .Arg<ffi::Buffer<ffi::U8>>()   // prepared parameters
                                  .Arg<ffi::Buffer<ffi::F32>>()  // electrons
                                  .Attr<int32_t>("n_up")
                                  .Attr<float>("cutoff")
                                  .Attr<float>("cutoff_1el")
                                  .Attr<int32_t>("cap_pairs")
                                  .Attr<int32_t>("cap_nuc")
                                  .Attr<int32_t>("precision")
                                  .Attr<int32_t>("chunk")
                                  .Ret<ffi::Buffer<ffi::F32>>()   // logpsi
                                  .Ret<ffi::Buffer<ffi::F32>>()   // sign
                                  .Ret<ffi::Buffer<ffi::F32>>()   // e_loc
                                  .Ret<ffi::Buffer<ffi::F64>>()   // (mean, std)
                                  .Ret<ffi::Buffer<ffi::S32>>());  // status words

XLA_FFI_DEFINE_HANDLER_SYMBOL(FireMcmcBlock, McmcBlock,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Ctx<ffi::ScratchAllocator>()
                                  .Arg<ffi::Buffer<ffi::F32>>()  // R
                                  .Arg<ffi::Buffer<ffi::F32>>()  // Z
                                  .Arg<ffi::Buffer<ffi::U8>>()   // prepared parameters
                                  .Arg<ffi::Buffer<ffi::F32>>()  // electrons
                                  .Arg<ffi::Buffer<ffi::F32>>()  // log|psi| of the electrons
                                  .Attr<int32_t>("n_up")
                                  .Attr<float>("cutoff")
                                  .Attr<float>("cutoff_1el")
                                  .Attr<int32_t>("cap_pairs")
                                  .Attr<int32_t>("cap_nuc")
                                  .Attr<int32_t>("precision")
                                  .Attr<int32_t>("chunk")
                                  .Attr<int32_t>("steps")
                                  .Attr<float>("width")
                                  .Attr<int64_t>("seed")
                                  .Attr<int64_t>("counter")
                                  .Ret<ffi::Buffer<ffi::F32>>()   // electrons after the block
                                  .Ret<ffi::Buffer<ffi::F32>>()   // log|psi| after the block
                                  .Ret<ffi::Buffer<ffi::S32>>()   // accepted moves per walker
                                  .Ret<ffi::Buffer<ffi::S32>>()   // static maxima [4]
                                  .Ret<ffi::Buffer<ffi::S32>>());  // status words

XLA_FFI_DEFINE_HANDLER_SYMBOL(FireLogpsiGrad, LogpsiGrad,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Ctx<ffi::ScratchAllocator>()
                                  .Arg<ffi::Buffer<ffi::F32>>()  // R
                                  .Arg<ffi::Buffer<ffi::U8>>()   // prepared parameters
                                  .Arg<ffi::Buffer<ffi::F32>>()  // electrons
                                  .Attr<int32_t>("n_up")
                                  .Attr<float>("cutoff")
                                  .Attr<float>("cutoff_1el")
                                  .Attr<int32_t>("cap_pairs")
                                  .Attr<int32_t>("cap_nuc")
                                  .Attr<int32_t>("chunk")
                                  .Ret<ffi::Buffer<ffi::F32>>()   // gradient rows [B, L]
                                  .Ret<ffi::Buffer<ffi::F32>>()   // logpsi
                                  .Ret<ffi::Buffer<ffi::F32>>()   // sign
                                  .Ret<ffi::Buffer<ffi::S32>>());  // status words
