// internal.h -- state shared by the library's translation units (not part
// of the C-ABI).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <mutex>
#include <string>

// one device and one stream; `scratch` is reusable device memory for calls
// that stage host arrays (the geometry sampling), grown on demand and freed
// with the context.  `relax_tune` caches the smoother autotuner's choice
// (colour cells per thread) per precision, h^2 form and level size class, so
// hierarchies uploaded later on the same context are not re-timed.
struct bsam_ctx_s {
  int device = 0;
  cudaStream_t stream = nullptr;
  void *scratch = nullptr;
  size_t scratch_bytes = 0;
  std::mutex tune_mu;
  std::map<uint64_t, int> relax_tune;
  // the context lives while it is open or a hierarchy made on it exists
  std::mutex ref_mu;
  int refs = 1;
};

// records the message of a failed call for bsam_last_error(); returns code
int bsam_internal_set_error(int code, const std::string &msg);
