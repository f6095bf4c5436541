// Library-wide C-ABI plumbing: version, thread-local last-error message.
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "common.cuh"

namespace tq {

static thread_local char g_err_msg[512] = "";
static thread_local int g_err_code = TQ_OK;

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err_msg, sizeof(g_err_msg), fmt, ap);
  va_end(ap);
  g_err_code = code;
  return code;
}

int cuda_status(cudaError_t e, const char* where) {
  snprintf(g_err_msg, sizeof(g_err_msg), "%s: CUDA error %d (%s)", where, (int)e,
           cudaGetErrorString(e));
  g_err_code = TQ_ERR_CUDA;
  return TQ_ERR_CUDA;
}

}  // namespace tq

extern "C" int tq_version(void) { return 100; }

extern "C" int tq_last_error(char* buf, size_t len) {
  if (buf && len > 0) {
    strncpy(buf, tq::g_err_msg, len - 1);
    buf[len - 1] = '\0';
  }
  return tq::g_err_code;
}
