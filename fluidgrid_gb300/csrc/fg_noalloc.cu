/* Allocation-free variant of the stable key/value radix sort.
 *
 * Some callers cannot allocate device memory when they sort: hosts that hand
 * the whole GPU to their own memory pool up front (a cudaMalloc from this
 * library could then fail or compete with the pool) and step loops that must
 * not stall, since the grow-only cache behind fgc_sort_pairs/gSort frees and
 * re-allocates (cudaFree waits for the device) whenever a larger sort
 * arrives.  fg_sort_pairs_noalloc sorts with scratch that lives in a
 * file-scope __device__ array instead, so it never calls cudaMalloc,
 * cudaFree or any allocating library routine.
 *
 * Limits and rules:
 *  - at most FG_NOALLOC_MAX_PAIRS (1,048,576) pairs per call; larger n is
 *    rejected with FG_E_INVALID and a message in fg_last_error();
 *  - the array (FG_NOALLOC_WORDS = 2,228,480 32-bit words: 8,913,920 bytes,
 *    8.91 MB or 8.5 MiB) is held on every GPU that loads this library until
 *    the process exits;
 *  - all calls share the array, so calls that overlap on the GPU (different
 *    streams, or several host threads) race and corrupt each other's results;
 *    serialise them;
 *  - every scratch word a call reads was written earlier by the same call, so
 *    nothing has to start at zero and the contents left by the previous call
 *    do not matter;
 *  - each call looks up the array's device address (cudaGetSymbolAddress
 *    with the caller's device current), so a context torn down and created
 *    again (cudaDeviceReset) is followed; while the stream is being captured
 *    the address cached by the last uncaptured call on that device is used
 *    instead, so the first call on a device must come before any stream
 *    capture;
 *  - an error left pending by earlier, unrelated work is cleared on entry, so
 *    FG_E_CUDA reports only this call's own launches and copies. */
#include <cuda_runtime.h>
#include <stdint.h>
#include <mutex>
#include "fg_kernels.h"
#include "fg_engine.h"
#include "../../include/fluidgrid_gb300.h"
#include "../../include/fluidgrid_reference.h"

#define FG_NOALLOC_MAX_PAIRS (1u << 20)
/* keys + values ping-pong buffers, then the radix tile histograms
 * (256 digits x one count per tile of FG_RS_TILE keys) and the 256 digit
 * totals */
#define FG_NOALLOC_HIST_WORDS (256u * ((FG_NOALLOC_MAX_PAIRS + FG_RS_TILE - 1u) / FG_RS_TILE) + 256u)
#define FG_NOALLOC_WORDS (2u * FG_NOALLOC_MAX_PAIRS + FG_NOALLOC_HIST_WORDS)

static __device__ __align__(256) uint32_t g_noalloc_scratch[FG_NOALLOC_WORDS];
static_assert(sizeof(g_noalloc_scratch) == 8913920u, "the documented scratch size is 8,913,920 bytes");

namespace {

const int kMaxDevices = 64;
uint32_t *g_scratch_ptr[kMaxDevices];
std::mutex g_setup_mu;

/* Device address of g_noalloc_scratch on the current device.  In host code
 * the symbol's name only stands for the array, it is not a device address.
 * Outside stream capture the address is looked up on every call (cheap), so
 * it follows a context that was reset and created again; while `stream` is
 * capturing, the address cached by the last uncaptured call is used. */
int scratch_for_current_device(cudaStream_t stream, uint32_t **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        fg::set_error("cudaGetDevice", e);
        return FG_E_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        fg::set_error_msg("fg_sort_pairs_noalloc: device ordinal out of range");
        return FG_E_UNSUPPORTED;
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(stream, &cs);
    if (e != cudaSuccess) {
        fg::set_error("cudaStreamIsCapturing", e);
        return FG_E_CUDA;
    }
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (cs != cudaStreamCaptureStatusNone) {
        if (!g_scratch_ptr[dev]) {
            fg::set_error_msg("fg_sort_pairs_noalloc: first call on this device made during stream capture");
            return FG_E_STATE;
        }
    } else {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            fg::set_error("cudaGetSymbolAddress(g_noalloc_scratch)", e);
            return FG_E_CUDA;
        }
        g_scratch_ptr[dev] = (uint32_t *)p;
    }
    *out = g_scratch_ptr[dev];
    return FG_OK;
}

} // namespace

extern "C" int fg_sort_pairs_noalloc(unsigned int *keys, unsigned int *values, unsigned int keyBits, unsigned int n,
                                     fg_stream_t stream)
{
    if (n == 0) return FG_OK;
    if (!keys || !values) {
        fg::set_error_msg("fg_sort_pairs_noalloc: null keys or values");
        return FG_E_INVALID;
    }
    if (n > FG_NOALLOC_MAX_PAIRS) {
        fg::set_error_msg("fg_sort_pairs_noalloc: n exceeds the allocation-free maximum of 1048576 pairs");
        return FG_E_INVALID;
    }
    if (keyBits > 32) keyBits = 32;
    uint32_t *s = nullptr;
    int r = scratch_for_current_device((cudaStream_t)stream, &s);
    if (r != FG_OK) return r;
    fg::RadixScratch rs;
    rs.keys_alt = s;
    rs.vals_alt = s + FG_NOALLOC_MAX_PAIRS;
    rs.hist = s + 2u * FG_NOALLOC_MAX_PAIRS;
    (void)cudaGetLastError(); /* only this call's own errors are reported below */
    cudaError_t e = fg::radix_sort(keys, values, keys, values, n, keyBits, 8, rs, (cudaStream_t)stream);
    const cudaError_t le = cudaGetLastError();
    if (e == cudaSuccess) e = le;
    if (e != cudaSuccess) {
        fg::set_error("fg_sort_pairs_noalloc", e);
        return FG_E_CUDA;
    }
    return FG_OK;
}
