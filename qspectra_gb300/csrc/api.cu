// Error plumbing and version of the qsx C ABI.
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "qsx_common.cuh"

namespace qsx {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int cuda_status(cudaError_t e, const char* where) {
  set_error("%s: CUDA error %d (%s)", where, (int)e, cudaGetErrorString(e));
  return QSX_ERR_CUDA;
}

}  // namespace qsx

extern "C" {

const char* qsx_last_error_string(void) { return qsx::g_err; }

int qsx_version(void) { return 100; }

}  // extern "C"
