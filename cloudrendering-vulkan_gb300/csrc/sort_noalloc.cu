// Radix sort entry point that allocates no device memory.
//
// Some callers cannot call cudaMalloc at the point where they need a sort:
// a host application that owns every device allocation through its own
// pool and forbids libraries from allocating, a real-time render loop that
// must not allocate (or free) after start-up because allocation can
// synchronise the device, or a plug-in that is handed device buffers and no
// allocator.  vcr_radix_sort_pairs_noalloc serves them: the caller passes
// the input and output buffers, and the sort's working memory (ping-pong
// copies, digit histograms, look-back words, tile counters, error word) is
// one file-scope device array that every GPU loading this library holds
// until the process exits.
//
// Limits and rules:
//  - at most VCR_SORT_NOALLOC_MAX_KEYS pairs per call (the array is sized
//    for that many: about 9.4 MB);
//  - all calls share the array, so calls whose work overlaps on the GPU
//    race with each other; serialise them (one stream, or events);
//  - the first call on each device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture;
//  - the array keeps the last call's contents; each call clears the parts
//    that must start at zero before its kernels run;
//  - a look-back wait that runs out sets the array's error word, which
//    vcr_sort_noalloc_status reads back and clears.
#include <mutex>

#include "vcr_internal.h"
#include "sort.cuh"

namespace vcr {

constexpr uint32_t kNoallocMaxKeys = VCR_SORT_NOALLOC_MAX_KEYS;
constexpr size_t kNoallocScratch = sort_scratch_bytes(kNoallocMaxKeys);

static __device__ __align__(256) unsigned char g_sort_scratch[kNoallocScratch];
static __device__ __align__(256) int g_sort_error;

namespace {

constexpr int kMaxDevices = 64;

// Device addresses of the two arrays, looked up once per device.  In host
// code the arrays' names are host-side stand-ins, never device addresses.
std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {};
int* g_error_ptr[kMaxDevices] = {};
int g_sm_count[kMaxDevices] = {};

cudaError_t setup_device(int dev) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_scratch_ptr[dev]) return cudaSuccess;
  void* s = nullptr;
  void* e = nullptr;
  cudaError_t r = cudaGetSymbolAddress(&s, g_sort_scratch);
  if (r != cudaSuccess) return r;
  r = cudaGetSymbolAddress(&e, g_sort_error);
  if (r != cudaSuccess) return r;
  int sms = 0;
  r = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (r != cudaSuccess) return r;
  g_sm_count[dev] = sms;
  g_error_ptr[dev] = static_cast<int*>(e);
  g_scratch_ptr[dev] = s;
  return cudaSuccess;
}

}  // namespace
}  // namespace vcr

using namespace vcr;

extern "C" VCR_API vcr_status vcr_radix_sort_pairs_noalloc(const uint32_t* d_keys_in, const uint32_t* d_vals_in,
                                                           uint32_t* d_keys_out, uint32_t* d_vals_out, uint32_t n,
                                                           uint32_t begin_bit, uint32_t end_bit, void* stream) {
  if (n > kNoallocMaxKeys)
    return fail(nullptr, VCR_ERR_CAPACITY,
                "vcr_radix_sort_pairs_noalloc: %u pairs exceed the fixed scratch of %u pairs; "
                "use vcr_radix_sort_pairs for larger sorts",
                n, kNoallocMaxKeys);
  if (n && (!d_keys_in || !d_keys_out || !d_vals_out))
    return fail(nullptr, VCR_ERR_INVALID, "vcr_radix_sort_pairs_noalloc: null buffer");
  if (begin_bit >= end_bit || end_bit > 32)
    return fail(nullptr, VCR_ERR_INVALID, "vcr_radix_sort_pairs_noalloc: bit range [%u, %u)", begin_bit, end_bit);
  if (d_vals_in == d_vals_out && d_keys_in != d_keys_out)
    return fail(nullptr, VCR_ERR_INVALID, "vcr_radix_sort_pairs_noalloc: values may alias only together with keys");
  if (n == 0) return VCR_OK;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(nullptr, VCR_ERR_UNSUPPORTED, "device ordinal %d", dev);
  e = setup_device(dev);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaGetSymbolAddress(sort scratch)");
  cudaStream_t st = (cudaStream_t)stream;
  e = cudaMemsetAsync(g_error_ptr[dev], 0, sizeof(int), st);
  if (e == cudaSuccess)
    e = sort_pairs_enqueue(g_sm_count[dev], g_error_ptr[dev], g_scratch_ptr[dev], d_keys_in, d_vals_in, d_keys_out,
                           d_vals_out, n, begin_bit, end_bit, st);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "vcr_radix_sort_pairs_noalloc");
  return VCR_OK;
}

// The sort's kernels set the device error word when a look-back wait runs
// out; this call is how a caller without a context learns of it.  It waits
// for the stream, copies the word into a host variable (no allocation) and
// clears it.
extern "C" VCR_API vcr_status vcr_sort_noalloc_status(void* stream) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(nullptr, VCR_ERR_UNSUPPORTED, "device ordinal %d", dev);
  e = setup_device(dev);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaGetSymbolAddress(sort error word)");
  cudaStream_t st = (cudaStream_t)stream;
  int word = 0;
  e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaMemcpy(&word, g_error_ptr[dev], sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && word) e = cudaMemset(g_error_ptr[dev], 0, sizeof(int));
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "vcr_sort_noalloc_status");
  if (word)
    return fail(nullptr, VCR_ERR_TIMEOUT, "vcr_radix_sort_pairs_noalloc: device error word %d (a look-back wait ran out)",
                word);
  return VCR_OK;
}
