// jubik_convolve2d_noalloc: the FFT convolution of jubik_convolve2d for callers
// that may not allocate device memory.
//
// Some callers cannot call cudaMalloc: code running under a framework that
// owns every byte of device memory through its own pool (an XLA FFI handler,
// a caching allocator that has reserved the GPU), or a latency-critical loop
// where an allocation would synchronise the device.  This entry point takes
// all of its scratch -- the twiddle tables of both axes and the complex
// spectra of kernel and signal -- from one file-scope device array of fixed
// size (JUBIK_NOALLOC_SCRATCH_BYTES), held by every GPU that loads the library
// until the process exits.  It calls no cudaMalloc, cudaFree or allocating
// library routine.
//
// The array is shared by every call on a device and keeps the last call's
// contents; everything a call reads is first written by that call, so nothing
// needs clearing.  Calls that overlap on the GPU (different streams, or
// different host threads without ordering) use the same memory and race.
//
// Host code cannot pass the array's name to a kernel (on the host it is a
// stand-in, not a device address): the first call on each device, with that
// device current, looks the address up with cudaGetSymbolAddress and caches
// it.  That first call therefore performs set-up work and should come before
// any stream capture.  The cached address belongs to the device's current
// context: a caller that destroys it (cudaDeviceReset) must not call this entry
// point again in the same process.
#include <cstdio>
#include <mutex>

#include "internal.h"
#include "jubik_common.cuh"

namespace jubik {
namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[JUBIK_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {nullptr};

size_t align256(size_t n) { return (n + 255) & ~size_t(255); }

// device address of the scratch array on the current device (cached per device)
int scratch_address(void** out) {
  int dev = 0;
  JUBIK_TRY_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("device ordinal %d beyond %d", dev, kMaxDevices);
    return JUBIK_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    JUBIK_TRY_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return JUBIK_OK;
}

}  // namespace
}  // namespace jubik

using namespace jubik;

extern "C" {

int jubik_convolve2d_noalloc(const void* kernel, int64_t bk, const void* signal, int64_t bs,
                             int32_t h, int32_t w, double dvol, int32_t dtype, void* out,
                             void* stream) {
  if (!kernel || !signal || !out || bk < 1 || bs < 1 || h < 1 || w < 1 || bs % bk != 0 ||
      (dtype != JUBIK_F32 && dtype != JUBIK_F64)) {
    set_error("convolve2d_noalloc: invalid arguments (kernel batch must divide the signal batch)");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  if (!fft_length_supported(h) || !fft_length_supported(w)) {
    set_error("convolve2d_noalloc: FFT size %d x %d unsupported", h, w);
    return JUBIK_ERR_UNSUPPORTED;
  }
  // scratch layout: twiddles (h, then w: float2 then double2), kernel spectra, signal spectra
  const size_t csz = dtype == JUBIK_F32 ? sizeof(float2) : sizeof(double2);
  const size_t hw = (size_t)h * (size_t)w;  // h, w <= 4096: no overflow
  // bound the plane counts before multiplying, so that no product wraps
  const size_t max_planes = (size_t)JUBIK_NOALLOC_SCRATCH_BYTES / (csz * hw);
  if ((uint64_t)bk > max_planes || (uint64_t)bs > max_planes) {
    set_error("convolve2d_noalloc: %lld kernel and %lld signal planes of %d x %d exceed the "
              "static scratch of %d bytes (use jubik_convolve2d)",
              (long long)bk, (long long)bs, h, w, JUBIK_NOALLOC_SCRATCH_BYTES);
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  const size_t tw_h32 = 0;
  const size_t tw_h64 = tw_h32 + align256(sizeof(float2) * h);
  const size_t tw_w32 = tw_h64 + align256(sizeof(double2) * h);
  const size_t tw_w64 = tw_w32 + align256(sizeof(float2) * w);
  const size_t zk_off = tw_w64 + align256(sizeof(double2) * w);
  const size_t zs_off = zk_off + align256(csz * hw * (size_t)bk);
  const size_t need = zs_off + align256(csz * hw * (size_t)bs);
  if (need > (size_t)JUBIK_NOALLOC_SCRATCH_BYTES) {
    set_error("convolve2d_noalloc: %zu bytes of scratch needed, the static scratch holds %d "
              "bytes (use fewer or smaller planes, or jubik_convolve2d)",
              need, JUBIK_NOALLOC_SCRATCH_BYTES);
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  void* base = nullptr;
  JUBIK_TRY(scratch_address(&base));
  unsigned char* b = static_cast<unsigned char*>(base);
  cudaStream_t s = (cudaStream_t)stream;
  Fft1D fh, fw;
  JUBIK_TRY(fft1d_init_external(&fh, h, b + tw_h32, b + tw_h64, s));
  JUBIK_TRY(fft1d_init_external(&fw, w, b + tw_w32, b + tw_w64, s));
  return dtype == JUBIK_F32
             ? convolve2d_run<float>(kernel, bk, signal, bs, (int64_t)hw, dvol, fh, fw,
                                     b + zk_off, b + zs_off, out, s)
             : convolve2d_run<double>(kernel, bk, signal, bs, (int64_t)hw, dvol, fh, fw,
                                      b + zk_off, b + zs_off, out, s);
}

}  // extern "C"
