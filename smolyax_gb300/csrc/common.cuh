// Shared helpers of the smolyax_gb300 CUDA library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/smolyax_gb300.h"

namespace smx {

// Records a message for smx_last_error_string() and returns `code`.
int set_error(int code, const std::string& msg);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Checks the last launch; returns SMX_OK or SMX_ERR_CUDA with a message.
int check_launch(const char* what);

inline unsigned int grid_for(int64_t n, int block) {
  int64_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > 0x7fffffff) g = 0x7fffffff;
  return static_cast<unsigned int>(g);
}

}  // namespace smx

#define SMX_REQUIRE(cond, msg)                                 \
  do {                                                         \
    if (!(cond)) return ::smx::set_error(SMX_ERR_ARG, (msg));  \
  } while (0)

#define SMX_LAUNCH_CHECK(what)                      \
  do {                                              \
    int _rc = ::smx::check_launch(what);            \
    if (_rc != SMX_OK) return _rc;                  \
  } while (0)
