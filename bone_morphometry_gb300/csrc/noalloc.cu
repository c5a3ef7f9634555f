// bm_edt_sq_device_noalloc: the exact squared EDT without any device
// allocation, for callers that cannot call cudaMalloc.
//
// Who needs this: code that runs where allocating device memory is not
// allowed or not possible -- a host that hands this library a fixed memory
// budget owned by its own pool allocator, a caller that must not change the
// device's memory footprint after start-up (real-time or certified pipelines),
// or an embedding that links the library into a process whose allocator it
// does not control.  bm_edt_sq_device draws its working buffers from a
// context's cache, which grows with cudaMalloc; this variant instead keeps all
// of its scratch in one file-scope __device__ array of fixed size, reserved
// when the library's module is loaded on a device and held until the process
// exits.
//
// Limits and behaviour (also stated in include/bm.h):
//  * scratch capacity kNoAllocScratchBytes = 32 MiB: volumes of up to about
//    2.7 million voxels (128^3 fits); larger volumes are rejected with
//    BM_ERR_DIMS before anything is launched;
//  * every call looks up the array's device address on the current device
//    with cudaGetSymbolAddress (which allocates nothing), so a
//    cudaDeviceReset between calls cannot leave a stale address behind; the
//    first call on a device also loads the library's device code there (lazy
//    module loading), so make that first call before any stream capture;
//  * every call on a device uses the same array and leaves its contents
//    behind; the counters that must start at zero are cleared with
//    cudaMemsetAsync on each call; calls whose work overlaps on the GPU (other
//    threads, other streams) race on the array and must be serialised by the
//    caller;
//  * no cudaMalloc, cudaFree or allocating library routine is called.
#include <cstdarg>
#include <cstdio>

#include "kernels.h"

namespace bm {
void set_thread_error(const char* msg);  // api.cu: message for bm_last_error(NULL, ...)
}

namespace {

constexpr size_t kNoAllocScratchBytes = 32u << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// The device address of the array on the current device.  Looked up on every
// call rather than cached: the lookup allocates nothing, and an address kept
// from before a cudaDeviceReset would point into a context that no longer
// exists.
cudaError_t scratch_for_current_device(void** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return e;
  *out = p;
  return cudaSuccess;
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

int fail_msg(int status, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int fail_msg(int status, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  bm::set_thread_error(buf);
  return status;
}

}  // namespace

extern "C" int bm_edt_sq_device_noalloc(const uint8_t* d_volume, size_t width, size_t height, size_t depth,
                                        int phase, uint32_t* d_out, void* stream) {
  using namespace bm;
  set_thread_error("");
  if (!d_volume || !d_out) return fail_msg(BM_ERR_INVALID, "null pointer");
  if (phase != BM_PHASE_FOREGROUND && phase != BM_PHASE_BACKGROUND)
    return fail_msg(BM_ERR_INVALID, "phase must be 0 (foreground) or 1 (background); got %d", phase);
  if (width < 2 || height < 2 || depth < 2)
    return fail_msg(BM_ERR_DIMS, "all dimensions must be at least 2 for 3-D morphometry; got %zux%zux%zu", width,
                    height, depth);
  if (width > 32768 || height > 32768 || depth > 32768)
    return fail_msg(BM_ERR_DIMS, "dimension above 32768 is not supported; got %zux%zux%zu", width, height, depth);
  const Dims dm{(int)width, (int)height, (int)depth};
  const size_t n = (size_t)dm.n();
  // scratch layout: counters | selection bits | y-pass map (u32) | envelope stack
  const size_t off_bits = align256(sizeof(Counters));
  const size_t bits_bytes = (size_t)dm.nw() * dm.h * dm.d * sizeof(uint32_t);
  const size_t off_map = off_bits + align256(bits_bytes);
  const size_t off_stack = off_map + align256(n * sizeof(uint32_t));
  const size_t need = off_stack + align256(edt_scratch_bytes(dm));
  if (n > (size_t)0xFFFFFFFFu || need > kNoAllocScratchBytes)
    return fail_msg(BM_ERR_DIMS,
                    "volume %zux%zux%zu needs %zu bytes of scratch; the no-allocation EDT holds %zu bytes "
                    "(about 2.7 million voxels)",
                    width, height, depth, need, kNoAllocScratchBytes);

  void* base = nullptr;
  cudaError_t e = scratch_for_current_device(&base);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail_msg(BM_ERR_CUDA, "scratch lookup: %s", cudaGetErrorString(e));
  }
  unsigned char* sb = static_cast<unsigned char*>(base);
  Counters* ctr = reinterpret_cast<Counters*>(sb);
  uint32_t* selbits = reinterpret_cast<uint32_t*>(sb + off_bits);
  uint32_t* ymap = reinterpret_cast<uint32_t*>(sb + off_map);
  void* stack = sb + off_stack;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned long long launches = 0;

  e = cudaMemsetAsync(ctr, 0, sizeof(Counters), s);  // the array keeps the last call's counters
  if (e == cudaSuccess)
    e = launch_edt_x(d_volume, nullptr, phase == BM_PHASE_BACKGROUND ? SEL_BACKGROUND : SEL_FOREGROUND, dm, d_out,
                     selbits, ctr, s, &launches);
  if (e == cudaSuccess) e = launch_edt_line(1, d_out, ymap, dm, stack, ctr, s, &launches);
  if (e == cudaSuccess) e = launch_edt_line(2, ymap, d_out, dm, stack, ctr, s, &launches);
  Counters hc{};
  if (e == cudaSuccess) e = cudaMemcpyAsync(&hc, ctr, sizeof hc, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail_msg(BM_ERR_CUDA, "no-allocation EDT: %s", cudaGetErrorString(e));
  }
  if (hc.sites == 0)
    return fail_msg(BM_ERR_ALL_SELECTED,
                    "distance transform is undefined for an all-%s volume unless an exterior convention is specified",
                    phase == BM_PHASE_BACKGROUND ? "background" : "foreground");
  return BM_OK;
}
