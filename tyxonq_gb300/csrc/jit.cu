// Runtime compilation of circuit-specialised pass kernels (NVRTC) and their
// launches.
//
// tyxonq_gb300/jit.py writes CUDA source for each register-staged forward
// pass of a circuit structure (straight-line register code per stage, see
// jit_staged.cuh).  tq_jit_build compiles one such source for sm_103a in
// process with NVRTC and hands back the cubin (the host side caches it on
// disk); tq_jit_load loads a cubin as a CUDA library and keeps its kernel.
// tq_jit_run_staged compiles the program's op records once (k_rops_compile,
// the same rop_build as the library's interpreting kernel) and launches every
// pass with its specialised kernel, or with the interpreting kernel
// (tq_sv_run_staged) where the host gave none.
#include <nvrtc.h>

#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "staged_io.cuh"
#include "wave_io.cuh"

namespace tq {

struct JitKernel {
  cudaLibrary_t lib = nullptr;
  cudaKernel_t kernel = nullptr;
};

static int nvrtc_fail(nvrtcResult r, const char* where) {
  return fail(TQ_ERR_CUDA, "%s: %s", where, nvrtcGetErrorString(r));
}

template <typename R>
static size_t jit_smem_bytes(int t, int nlow, int nops, int dbuf) {
  return (size_t)(dbuf ? 2 : 1) * padded_len(t) * sizeof(cplx<R>) + staged_hoff_bytes(t, nlow) +
         (size_t)nops * sizeof(ROp<R>);
}

// Forward op records of the whole op table (one thread per op).
template <typename R>
__global__ void k_rops_compile(ROp<R>* out, const tq_tile_op* __restrict__ ops, int n_ops,
                               const double* __restrict__ theta) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n_ops) rop_build<R>(out[k], ops, k, theta, false, false);
}

// Op records of wave passes: one CTA per job, one thread per op.
template <typename R>
__global__ void k_wave_rops(const tq_rop_job* __restrict__ jobs, int n_jobs, const tq_tile_op* __restrict__ ops,
                            const double* __restrict__ theta, ROp<R>* out) {
  for (int j = blockIdx.x; j < n_jobs; j += gridDim.x) {
    const tq_rop_job J = jobs[j];
    const bool adj = (J.flags & 1) != 0;
    for (int k = threadIdx.x; k < J.n_ops; k += blockDim.x)
      rop_build<R>(out[J.out_record + k], ops, J.op_begin + k, theta + J.theta_off, adj, adj);
  }
}

}  // namespace tq

using namespace tq;

extern "C" int tq_jit_build(const char* source, const char* const* include_dirs, int n_include_dirs, void** cubin,
                            size_t* cubin_size, char* log, size_t log_cap) {
  TQ_RANGE("tq_jit_build");
  if (!source || !cubin || !cubin_size) return fail(TQ_ERR_ARG, "tq_jit_build: NULL argument");
  *cubin = nullptr;
  *cubin_size = 0;
  if (log && log_cap) log[0] = 0;
  nvrtcProgram prog;
  nvrtcResult r = nvrtcCreateProgram(&prog, source, "tq_jit.cu", 0, nullptr, nullptr);
  if (r != NVRTC_SUCCESS) return nvrtc_fail(r, "tq_jit_build: nvrtcCreateProgram");
  // unannotated declarations of the C ABI header are device-side in runtime compilation
  std::vector<std::string> opts = {"-arch=sm_103a", "-std=c++17", "-lineinfo", "-default-device"};
  for (int i = 0; i < n_include_dirs; ++i)
    if (include_dirs && include_dirs[i]) opts.push_back(std::string("--include-path=") + include_dirs[i]);
  std::vector<const char*> copts;
  for (auto& o : opts) copts.push_back(o.c_str());
  r = nvrtcCompileProgram(prog, (int)copts.size(), copts.data());
  if (r != NVRTC_SUCCESS) {
    size_t n = 0;
    nvrtcGetProgramLogSize(prog, &n);
    std::string msg(n, '\0');
    if (n) nvrtcGetProgramLog(prog, &msg[0]);
    if (log && log_cap) {
      const size_t k = msg.size() < log_cap - 1 ? msg.size() : log_cap - 1;
      msg.copy(log, k);
      log[k] = 0;
    }
    nvrtcDestroyProgram(&prog);
    return fail(TQ_ERR_CUDA, "tq_jit_build: NVRTC compilation failed (%s): %.300s", nvrtcGetErrorString(r),
                msg.c_str());
  }
  size_t size = 0;
  r = nvrtcGetCUBINSize(prog, &size);
  if (r != NVRTC_SUCCESS || size == 0) {
    nvrtcDestroyProgram(&prog);
    return nvrtc_fail(r, "tq_jit_build: nvrtcGetCUBINSize");
  }
  void* buf = std::malloc(size);
  if (!buf) {
    nvrtcDestroyProgram(&prog);
    return fail(TQ_ERR_RANGE, "tq_jit_build: no host memory for a %zu-byte cubin", size);
  }
  r = nvrtcGetCUBIN(prog, static_cast<char*>(buf));
  nvrtcDestroyProgram(&prog);
  if (r != NVRTC_SUCCESS) {
    std::free(buf);
    return nvrtc_fail(r, "tq_jit_build: nvrtcGetCUBIN");
  }
  *cubin = buf;
  *cubin_size = size;
  return TQ_OK;
}

extern "C" void tq_jit_free_host(void* p) { std::free(p); }

extern "C" int tq_jit_load(const void* cubin, size_t cubin_size, const char* kernel_name, void** kernel_out) {
  if (!cubin || !cubin_size || !kernel_name || !kernel_out) return fail(TQ_ERR_ARG, "tq_jit_load: NULL argument");
  *kernel_out = nullptr;
  JitKernel* k = new JitKernel();
  cudaError_t e = cudaLibraryLoadData(&k->lib, cubin, nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (e != cudaSuccess) {
    delete k;
    return cuda_status(e, "tq_jit_load: cudaLibraryLoadData");
  }
  e = cudaLibraryGetKernel(&k->kernel, k->lib, kernel_name);
  if (e != cudaSuccess) {
    cudaLibraryUnload(k->lib);
    delete k;
    return fail(TQ_ERR_CUDA, "tq_jit_load: kernel '%s' not found: %s", kernel_name, cudaGetErrorString(e));
  }
  *kernel_out = k;
  return TQ_OK;
}

extern "C" int tq_jit_unload(void* kernel) {
  if (!kernel) return TQ_OK;
  JitKernel* k = static_cast<JitKernel*>(kernel);
  cudaError_t e = cudaLibraryUnload(k->lib);
  delete k;
  return e == cudaSuccess ? TQ_OK : cuda_status(e, "tq_jit_unload");
}

extern "C" size_t tq_jit_rops_bytes(int dtype, int n_ops) {
  return (size_t)(n_ops > 0 ? n_ops : 0) * (dtype == TQ_C64 ? sizeof(ROp<float>) : sizeof(ROp<double>));
}

extern "C" int tq_sv_run_staged(void* psi, int n, int dtype, const tq_tile_pass* passes, int n_passes,
                                const tq_tile_stage* stages, const tq_tile_op* ops, const double* theta,
                                void* stream);

extern "C" int tq_jit_run_staged(void* const* kernels, int stage_bits, void* psi, int n, int dtype,
                                 const tq_tile_pass* passes,
                                 int n_passes, const tq_tile_stage* stages_host, const tq_tile_stage* stages,
                                 const tq_tile_op* ops, int n_ops, const double* theta, void* ws, size_t ws_bytes,
                                 void* stream) {
  TQ_RANGE("tq_jit_run_staged");
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if (n_passes <= 0) return TQ_OK;
  if (!kernels || !passes || !stages_host || !stages || !ops || !psi)
    return fail(TQ_ERR_ARG, "tq_jit_run_staged: NULL argument");
  if (n_ops <= 0) return fail(TQ_ERR_ARG, "tq_jit_run_staged: empty op table");
  if (stage_bits != 4 && stage_bits != 5)
    return fail(TQ_ERR_ARG, "tq_jit_run_staged: %d register bits per stage (4 or 5)", stage_bits);
  const size_t need = tq_jit_rops_bytes(dtype, n_ops);
  if (!ws || ws_bytes < need)
    return fail(TQ_ERR_WORKSPACE, "tq_jit_run_staged: workspace of %zu bytes, %zu needed", ws_bytes, need);
  if ((reinterpret_cast<uintptr_t>(ws) & 15) != 0) return fail(TQ_ERR_ARG, "tq_jit_run_staged: workspace not 16-byte aligned");
  // 5-bit stages hold twice the amplitudes per thread: one more tile bit
  const int tmax = (dtype == TQ_C64 ? 13 : 12) + (stage_bits == 5 ? 1 : 0);
  for (int p = 0; p < n_passes; ++p) {
    const tq_tile_pass& tp = passes[p];
    if (tp.op_end == tp.op_begin) continue;
    if (!kernels[p]) {
      if (stage_bits != 4)
        return fail(TQ_ERR_ARG, "tq_jit_run_staged: pass %d has no kernel and %d-bit stages", p, stage_bits);
      continue;
    }
    if (tp.t < 9 || tp.t > tmax || tp.t > n || tp.nlow < 1 || tp.nlow > tp.t || tp.t - stage_bits < 5)
      return fail(TQ_ERR_ARG, "tq_jit_run_staged: pass %d has t=%d nlow=%d (n=%d)", p, tp.t, tp.nlow, n);
    const int op0 = stages_host[tp.op_begin].op_begin, op1 = stages_host[tp.op_end - 1].op_end;
    if (op0 < 0 || op1 > n_ops || op1 - op0 <= 0 || op1 - op0 > kStagedRopCap)
      return fail(TQ_ERR_RANGE, "tq_jit_run_staged: pass %d has ops [%d, %d) (table %d, at most %d per pass)", p,
                  op0, op1, n_ops, kStagedRopCap);
  }
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned cb = (unsigned)((n_ops + 127) / 128);
  if (dtype == TQ_C64)
    k_rops_compile<float><<<cb, 128, 0, s>>>(static_cast<ROp<float>*>(ws), ops, n_ops, theta);
  else
    k_rops_compile<double><<<cb, 128, 0, s>>>(static_cast<ROp<double>*>(ws), ops, n_ops, theta);
  TQ_CHECK_LAUNCH("tq_jit_run_staged: op records");
  for (int p = 0; p < n_passes; ++p) {
    const tq_tile_pass& tp = passes[p];
    if (tp.op_end == tp.op_begin) continue;
    if (!kernels[p]) {  // the interpreting kernel for this pass
      rc = tq_sv_run_staged(psi, n, dtype, &tp, 1, stages, ops, theta, stream);
      if (rc) return rc;
      continue;
    }
    PassArgs P;
    P.n = n;
    P.t = tp.t;
    P.nlow = tp.nlow;
    P.op_begin = tp.op_begin;
    P.op_end = tp.op_end;
    for (int i = 0; i < TQ_TILE_MAX_BITS; ++i) P.pos[i] = tp.pos[i];
    const int nops = stages_host[tp.op_end - 1].op_end - stages_host[tp.op_begin].op_begin;
    const int threads = 1 << (tp.t - stage_bits);
    const int64_t ntiles = int64_t(1) << (n - tp.t);
    cudaKernel_t k = static_cast<JitKernel*>(kernels[p])->kernel;
    // Buffering: double (the next tile streams in while a CTA computes) unless
    // single buffers let more CTAs share an SM (then resident CTAs overlap each
    // other's loads) or every CTA owns one tile.
    const size_t smem1 = dtype == TQ_C64 ? jit_smem_bytes<float>(tp.t, tp.nlow, nops, 0)
                                         : jit_smem_bytes<double>(tp.t, tp.nlow, nops, 0);
    const size_t smem2 = dtype == TQ_C64 ? jit_smem_bytes<float>(tp.t, tp.nlow, nops, 1)
                                         : jit_smem_bytes<double>(tp.t, tp.nlow, nops, 1);
    if (smem1 > 227 * 1024)
      return fail(TQ_ERR_ARG, "tq_jit_run_staged: pass %d needs %zu bytes of shared memory", p, smem1);
    const bool dbuf_fits = smem2 <= 227 * 1024;
    cudaError_t e = cudaKernelSetAttributeForDevice(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    (int)(dbuf_fits ? smem2 : smem1), dev);
    if (e != cudaSuccess) return cuda_status(e, "tq_jit_run_staged: shared memory attribute");
    int occ1 = 1, occ2 = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ1, (const void*)k, threads, smem1);
    if (e == cudaSuccess && dbuf_fits) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ2, (const void*)k, threads, smem2);
    if (e != cudaSuccess) return cuda_status(e, "tq_jit_run_staged: occupancy");
    if (occ1 < 1) occ1 = 1;
    int dbuf = (dbuf_fits && occ2 >= 1 && occ2 >= occ1 && ntiles > (int64_t)sms * occ2) ? 1 : 0;
    const int occ = dbuf ? occ2 : occ1;
    const size_t smem = dbuf ? smem2 : smem1;
    const int64_t cap = (int64_t)sms * occ;
    const unsigned grid = (unsigned)(ntiles < cap ? ntiles : cap);
    void* rops = ws;
    void* args[] = {&psi, &n, &P, (void*)&stages, (void*)&ops, &rops, &dbuf};
    e = cudaLaunchKernel((const void*)k, dim3(grid), dim3(threads), args, smem, s);
    if (e != cudaSuccess) return cuda_status(e, "tq_jit_run_staged: launch");
  }
  return TQ_OK;
}

extern "C" int tq_wave_rops(int dtype, const tq_rop_job* jobs, int n_jobs, const tq_tile_op* ops, const double* theta,
                            void* out, void* stream) {
  TQ_RANGE("tq_wave_rops");
  if (dtype != TQ_C64 && dtype != TQ_C128) return fail(TQ_ERR_ARG, "tq_wave_rops: dtype tag %d", dtype);
  if (n_jobs < 0) return fail(TQ_ERR_ARG, "tq_wave_rops: negative job count");
  if (n_jobs == 0) return TQ_OK;
  if (!jobs || !ops || !theta || !out) return fail(TQ_ERR_ARG, "tq_wave_rops: NULL argument");
  if ((reinterpret_cast<uintptr_t>(out) & 15) != 0) return fail(TQ_ERR_ARG, "tq_wave_rops: output not 16-byte aligned");
  const unsigned grid = (unsigned)(n_jobs < 152 * 16 ? n_jobs : 152 * 16);
  if (dtype == TQ_C64)
    k_wave_rops<float><<<grid, 128, 0, (cudaStream_t)stream>>>(jobs, n_jobs, ops, theta, (ROp<float>*)out);
  else
    k_wave_rops<double><<<grid, 128, 0, (cudaStream_t)stream>>>(jobs, n_jobs, ops, theta, (ROp<double>*)out);
  TQ_CHECK_LAUNCH("tq_wave_rops");
  return TQ_OK;
}

extern "C" int tq_jit_wave_run(void* kernel, int kind, int dtype, const tq_wave_item* items, int n_items, int t,
                               const tq_tile_pass* passes, const tq_tile_stage* stages, const tq_tile_op* ops,
                               const double* theta, const void* rops, void* pool, double* partials, int max_ops,
                               void* stream) {
  TQ_RANGE("tq_jit_wave_run");
  if (!kernel || !items || !passes || !stages || !ops || !pool || (kind == 2 && !partials))
    return fail(TQ_ERR_ARG, "tq_jit_wave_run: NULL argument");
  if (kind != 0 && kind != 2) return fail(TQ_ERR_ARG, "tq_jit_wave_run: kind %d (0 forward, 2 adjoint)", kind);
  if (dtype != TQ_C64 && dtype != TQ_C128) return fail(TQ_ERR_ARG, "tq_jit_wave_run: dtype tag %d", dtype);
  if (t < 9 || t > (dtype == TQ_C64 ? 13 : 12)) return fail(TQ_ERR_ARG, "tq_jit_wave_run: t=%d", t);
  if (max_ops < 1 || max_ops > 4096) return fail(TQ_ERR_ARG, "tq_jit_wave_run: max_ops %d", max_ops);
  if (n_items <= 0) return TQ_OK;
  const size_t S = dtype == TQ_C64 ? sizeof(cplx<float>) : sizeof(cplx<double>);
  const size_t rop = dtype == TQ_C64 ? sizeof(ROp<float>) : sizeof(ROp<double>);
  const size_t R = dtype == TQ_C64 ? sizeof(float) : sizeof(double);
  const int threads = 1 << (t - kRB);
  size_t smem = (kind == 0 ? 1 : 2) * padded_len(t) * S + w_hoff_bytes(t) + (size_t)max_ops * rop;
  if (kind == 2) smem += R * (size_t)max_ops * (threads / 32);
  if (smem > 227 * 1024) return fail(TQ_ERR_ARG, "tq_jit_wave_run: %zu bytes of shared memory", smem);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e, "tq_jit_wave_run: device");
  cudaKernel_t k = static_cast<JitKernel*>(kernel)->kernel;
  e = cudaKernelSetAttributeForDevice(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem, dev);
  if (e != cudaSuccess) return cuda_status(e, "tq_jit_wave_run: shared memory attribute");
  if (rops && (reinterpret_cast<uintptr_t>(rops) & 15) != 0)
    return fail(TQ_ERR_ARG, "tq_jit_wave_run: op records not 16-byte aligned");
  void* args_f[] = {(void*)&items, &n_items, (void*)&passes, (void*)&stages, (void*)&ops, (void*)&theta,
                    (void*)&rops, &pool, &max_ops};
  void* args_a[] = {(void*)&items, &n_items, (void*)&passes, (void*)&stages, (void*)&ops, (void*)&theta,
                    (void*)&rops, &pool, (void*)&partials, &max_ops};
  e = cudaLaunchKernel((const void*)k, dim3((unsigned)n_items), dim3(threads), kind == 0 ? args_f : args_a, smem,
                       (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_status(e, "tq_jit_wave_run: launch");
  return TQ_OK;
}

