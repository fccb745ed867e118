// af_noalloc.cu -- a power-of-two transform entry point that allocates no
// device memory.
//
// Some callers cannot call cudaMalloc: code that runs inside a memory pool
// or arena owned by someone else, callers that must not touch the CUDA
// allocator while other work is being captured or timed, and embedders that
// forbid allocation after start-up.  For them, af_exec_c2c_noalloc runs the
// same split-radix / four-step tile program as af_exec_c2c for power-of-two
// lengths, but its scratch workspace, twiddle tables and launch descriptors
// live in the file-scope device arrays below.  Every GPU that loads libaf
// holds these arrays (about 19 MiB) until the process exits.
//
// The first call on a device looks the arrays up with cudaGetSymbolAddress
// (once per device, with that device current).  Every call uploads its launch
// descriptors from host memory, so no call can be captured in a CUDA graph: a
// call on a capturing stream fails with AF_ERR_UNSUPPORTED before it does
// anything.  All calls share the arrays and each call overwrites them, so
// calls that overlap on the GPU (on different streams) race; calls in one
// stream are ordered.
#include <mutex>

#include "af_host.h"

namespace af {

// Largest n * batch the scratch workspace holds: 2^21 complex values (16 MiB).
static const i64 kNoAllocMaxElems = (i64)1 << 21;
static const i64 kNoAllocTables = 8192;         // float2 entries of twiddle tables
static const i64 kNoAllocBlob = (i64)2 << 20;   // bytes of descriptors and work items

// the workspace of a four-step program is n * batch plus alignment slack
static const i64 kNoAllocScratch = kNoAllocMaxElems + 4096;
static __device__ __align__(256) float2 g_scratch[kNoAllocScratch];
static __device__ __align__(256) float2 g_tables[kNoAllocTables];
static __device__ __align__(256) char g_blob[kNoAllocBlob];

struct NoAllocDevice {
  bool ready = false;
  float2* scratch = nullptr;
  float2* tables = nullptr;
  char* blob = nullptr;
};

static const int kMaxDevices = 64;
static NoAllocDevice g_devices[kMaxDevices];
static std::mutex g_mutex;

// Device addresses of the arrays for the current device (looked up once).
static void device_arrays(NoAllocDevice* out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) throw AfError(AF_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) throw AfError(AF_ERR_UNSUPPORTED, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_mutex);
  NoAllocDevice& d = g_devices[dev];
  if (!d.ready) {
    NoAllocDevice t;
    e = cudaGetSymbolAddress((void**)&t.scratch, g_scratch);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&t.tables, g_tables);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&t.blob, g_blob);
    if (e != cudaSuccess) {
      cudaGetLastError();
      throw AfError(AF_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    }
    t.ready = true;
    d = t;
  }
  *out = d;
}

}  // namespace af

using namespace af;

extern "C" af_status af_exec_c2c_noalloc(int64_t n, int sign, const float* in, float* out, int64_t batch,
                                         af_stream stream) {
  auto fail = [&](af_status code, const std::string& m) {
    set_last_error(m);
    return code;
  };
  try {
    if (n < 1 || (n & (n - 1))) return fail(AF_ERR_INVALID, "length must be a power of two");
    if (sign != 1 && sign != -1) return fail(AF_ERR_INVALID, "sign must be -1 (forward) or +1 (inverse)");
    if (batch < 0) return fail(AF_ERR_INVALID, "negative batch");
    // checked without forming n * batch, which could overflow
    if (n > kNoAllocMaxElems || batch > kNoAllocMaxElems / n)
      return fail(AF_ERR_INVALID, "n * batch (n = " + std::to_string(n) + ", batch = " + std::to_string(batch) +
                                      ") exceeds the static workspace of " + std::to_string(kNoAllocMaxElems) +
                                      " complex values");
    if (!in || !out) return fail(AF_ERR_INVALID, "null data pointer");
    if (((uintptr_t)in | (uintptr_t)out) & 7) return fail(AF_ERR_INVALID, "data must be 8-byte aligned");
    // each call uploads its launch descriptors from host memory, which a
    // stream capture cannot record: refuse before touching the stream
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaError_t ce = cudaStreamIsCapturing((cudaStream_t)stream, &cap);
    if (ce != cudaSuccess) return fail(AF_ERR_CUDA, std::string("cudaStreamIsCapturing: ") + cudaGetErrorString(ce));
    if (cap != cudaStreamCaptureStatusNone)
      return fail(AF_ERR_UNSUPPORTED, "af_exec_c2c_noalloc cannot be captured in a CUDA graph: each call uploads its "
                                      "launch descriptors from host memory");
    if (batch == 0) return AF_OK;
    NoAllocDevice dev;
    device_arrays(&dev);
    // plan tree and launch program on the host; tables and descriptors go to
    // the static arrays on the caller's stream
    Planner pl;
    const Node* root = pl.decompose(n);
    PlanRes res;
    res.no_alloc = true;
    res.arena = dev.tables;
    res.arena_cap = (size_t)kNoAllocTables;
    res.blob = dev.blob;
    res.blob_cap = (size_t)kNoAllocBlob;
    res.stream = (cudaStream_t)stream;
    Program prog;
    build_program(res, root, (float)sign, batch, &prog);
    if (prog.ws_elems > kNoAllocScratch) return fail(AF_ERR_UNSUPPORTED, "workspace exceeds the static array");
    TileBases b = make_bases(in, nullptr, out, nullptr, dev.scratch, nullptr, nullptr);
    const cudaError_t e = run_program(prog, b, nullptr, (cudaStream_t)stream);
    if (e != cudaSuccess) return fail(AF_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    return AF_OK;
  } catch (const AfError& e) {
    return fail(e.code, e.what());
  } catch (const std::exception& e) {
    return fail(AF_ERR_INVALID, e.what());
  }
}
