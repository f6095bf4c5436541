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

#ifdef TQ_CHECKED
extern "C" int tq_check_read_gates(unsigned long long* out);
extern "C" int tq_check_read_program(unsigned long long* out);
extern "C" int tq_check_read_wave(unsigned long long* out);
extern "C" int tq_check_read_measure(unsigned long long* out);
#endif

extern "C" int tq_check_status(unsigned* site, long long* index) {
  if (site) *site = 0;
  if (index) *index = 0;
#ifdef TQ_CHECKED
  int (*readers[])(unsigned long long*) = {tq_check_read_gates, tq_check_read_program, tq_check_read_wave,
                                           tq_check_read_measure};
  for (auto rd : readers) {
    unsigned long long w[2] = {0ull, 0ull};
    const int e = rd(w);
    if (e != 0) return tq::cuda_status((cudaError_t)e, "tq_check_status");
    if (w[0] != 0ull && site && *site == 0) {
      *site = (unsigned)w[0];
      if (index) *index = (long long)w[1];
    }
  }
  return 1;
#else
  return 0;
#endif
}
