// Reconstruction entry point that needs no workspace from the caller.
//
// Some callers cannot allocate device memory at all: a plugin running inside a host framework
// that has reserved the whole GPU for its own pool (a late cudaMalloc fails or fragments it),
// a real-time pipeline that forbids allocation once it is running, or a foreign-language host
// that only receives device buffers and has no allocator of its own to size a workspace with.
// nsgb_imreconstruct_noalloc serves them: its scratch is a fixed-size array in this library's
// own device memory, which every GPU that loads the library holds until the process exits.
//
// The scratch holds the reconstruction work queue (a status header, one state word per tile
// and the tile ring), so the limit is a number of tiles: see NSGB_NOALLOC_SCRATCH_BYTES in
// include/nsgb.h.  Every call clears what it uses before its kernel runs, but all calls share
// the one array: calls whose work overlaps on the GPU (other streams, other host threads)
// race on it and must be serialised by the caller.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/nsgb.h"
#include "common.cuh"
#include "recon.cuh"

namespace {

// File-scope scratch in device memory.  Host code must never pass `g_noalloc_scratch`
// itself to a kernel (on the host it is only a stand-in symbol); it uses the device address
// that cudaGetSymbolAddress returns.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NSGB_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch on the current device.  Outside stream capture it is looked up
// on every call (cheap: a table lookup in the runtime), so a context that was reset or
// re-created since the last call -- which loads the module again, possibly at another address
// -- is followed.  While `s` is capturing, the address recorded by the last call outside
// capture on this device is used (a lookup could load the module inside the capture); without
// one the call fails.
cudaError_t scratch_address(cudaStream_t s, void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  e = cudaStreamIsCapturing(s, &cap);
  const bool capturing = e != cudaSuccess || cap != cudaStreamCaptureStatusNone;
  if (e != cudaSuccess) (void)cudaGetLastError();  // e.g. the legacy stream during a global capture
  std::lock_guard<std::mutex> lock(g_mu);
  if (!capturing) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = p;
  }
  if (!g_scratch_ptr[dev]) return cudaErrorStreamCaptureUnsupported;
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" nsgb_status nsgb_imreconstruct_noalloc(int dtype, void* marker, const void* mask, int64_t rows,
                                                  int64_t cols, int64_t pitch, int conn, int erode,
                                                  nsgb_stream_t stream, const nsgb_opts* opts) {
  const int esz = nsgb::elem_size(dtype);
  if (!esz) return NSGB_ERR_UNSUPPORTED_DTYPE;
  if (!marker || !mask || !nsgb::valid_dims(rows, cols) || !nsgb::valid_pitch(pitch, cols, esz) ||
      !nsgb::valid_conn(conn))
    return NSGB_ERR_BAD_ARG;
  // Too large for the built-in scratch: refuse before touching the GPU.
  if (nsgb::recon_workspace_bytes(dtype, rows, cols) > (size_t)NSGB_NOALLOC_SCRATCH_BYTES)
    return NSGB_ERR_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  void* ws = nullptr;
  if (scratch_address(s, &ws) != cudaSuccess) return NSGB_ERR_CUDA;
  const bool ring = !erode && (dtype == NSGB_I32 || dtype == NSGB_F32);
  if (opts && opts->recon_event_begin && cudaEventRecord((cudaEvent_t)opts->recon_event_begin, s) != cudaSuccess)
    return NSGB_ERR_CUDA;
  cudaError_t e = nsgb::recon_launch(dtype, marker, marker, mask, rows, cols, pitch, conn, erode != 0, ring, ws, s,
                                     opts ? opts->max_visits_per_tile : 0, opts ? opts->max_visit_iters : 0,
                                     opts ? opts->queue_poll_limit : 0, opts ? opts->recon_passes : 0,
                                     opts ? opts->recon_order : 0, opts ? opts->recon_ctas_per_sm : 0);
  if (e != cudaSuccess) return NSGB_ERR_CUDA;
  if (opts && opts->recon_event_end && cudaEventRecord((cudaEvent_t)opts->recon_event_end, s) != cudaSuccess)
    return NSGB_ERR_CUDA;
  if (opts && !opts->sync) return NSGB_OK;
  return nsgb_noalloc_device_status(stream);
}

// Reads the device status word at the start of the built-in scratch, after the work already on
// `stream`: the status of the last nsgb_imreconstruct_noalloc call on this device, as long as
// no later call has started (each call resets it).
extern "C" nsgb_status nsgb_noalloc_device_status(nsgb_stream_t stream) {
  cudaStream_t s = (cudaStream_t)stream;
  void* ws = nullptr;
  if (scratch_address(s, &ws) != cudaSuccess) return NSGB_ERR_CUDA;
  int dev_status = 0;
  if (cudaMemcpyAsync(&dev_status, ws, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return NSGB_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return NSGB_ERR_CUDA;
  return (nsgb_status)dev_status;
}
