// Batched log density and gradient without any device allocation.
//
// Who needs this: code that may not call cudaMalloc at the moment it needs a
// gradient, for example a host that has reserved all device memory up front
// for its own pool, a callback running inside another framework's allocator
// lock, or a latency-critical loop where an allocation (and the implicit
// synchronisation it can cause) is not acceptable.  The regular batched entry
// point grows a workspace owned by the model handle with cudaMalloc on first
// use and whenever the chain count changes; this one never does.
//
// The scratch it needs (per row split and chain: the partial sums of lp and of
// the gradient; per chain and group: the group sums; the split boundaries and
// an error flag) lives in one file-scope device array of fixed size,
// kNoAllocScratchBytes.  Every GPU that loads the library holds that array
// until the process exits.  All calls on a device share it and it keeps the
// last call's contents, so the parts that must start at zero are cleared on
// every call, and two calls that overlap on the GPU (different streams, or
// different host threads without ordering) race on it.
//
// The device address of the array is obtained once per device, with that
// device current, on the first call made on that device; that first call
// should therefore be made before any stream capture begins.  The address is
// kept for the life of the process: a device reset (which discards the
// module and its array) is not supported while the library is loaded.
//
// Per call, a one-thread-block kernel writes the split boundaries and clears
// the error flag inside the array (nothing is copied from host memory), then
// the gradient kernels of the regular entry point run on the same stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "../../include/gbnuts.h"
#include "gbnuts_internal.h"

namespace gbn {

// 16 MiB: enough for, e.g., 1024 chains x K = 100 x 19 row splits, or 256
// chains of a 2000-group hierarchical model.
constexpr size_t kNoAllocScratchBytes = 16u << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {nullptr};

// Once per device, with that device current: the device address of the array.
int scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_last_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    return GBNUTS_SOFTWARE;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    set_last_error("device index beyond the no-allocation entry point's table");
    return GBNUTS_SOFTWARE;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      set_last_error(std::string("cudaGetSymbolAddress of the scratch array: ") +
                     cudaGetErrorString(e));
      return GBNUTS_SOFTWARE;
    }
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return GBNUTS_OK;
}

size_t align256(size_t n) { return (n + 255) & ~(size_t)255; }
}  // namespace

// Split boundaries for S splits of N rows (rows[s] = N s / S), or for a
// hierarchical model the first row of group J s / S (rows sorted by group,
// so that is the count of rows whose group is below it), and a cleared
// error flag.
__global__ void noalloc_setup_kernel(long long N, int S, int J, const int* __restrict__ group,
                                     long long* __restrict__ rows, int* __restrict__ err) {
  for (int s = threadIdx.x; s <= S; s += blockDim.x) {
    long long r;
    if (group == nullptr) {
      r = N * s / S;
    } else {
      const long long j = (long long)J * s / S;
      long long lo = 0, hi = N;
      while (lo < hi) {
        const long long mid = lo + (hi - lo) / 2;
        if (group[mid] < j)
          lo = mid + 1;
        else
          hi = mid;
      }
      r = lo;
    }
    rows[s] = r;
  }
  if (threadIdx.x == 0) *err = 0;
}

}  // namespace gbn

// Reads the model descriptor and the host copy of the group offsets; declared
// in capi.cu beside the model handle.
int gbnuts_internal_model_view(const gbnuts_model* m, gbn::ModelDesc* desc,
                               const int** group_off);

extern "C" int gbnuts_log_prob_grad_batch_device_noalloc(gbnuts_model* m, int C,
                                                         const double* d_theta, double* d_lp,
                                                         double* d_grad, int precision,
                                                         void* stream) {
  using namespace gbn;
  if (!m || C <= 0 || !d_theta || !d_lp || !d_grad) {
    set_last_error("bad arguments");
    return GBNUTS_USAGE;
  }
  if (precision != GBNUTS_PREC_FP64 && precision != GBNUTS_PREC_FP32) {
    set_last_error("the no-allocation entry point supports the fp64 and fp32 forms only");
    return GBNUTS_USAGE;
  }
  ModelDesc desc;
  const int* group_off = nullptr;
  int rc = gbnuts_internal_model_view(m, &desc, &group_off);
  if (rc) return rc;
  const int CB = chains_per_block(desc.K);
  if (CB == 0) {
    set_last_error("K beyond the supported maximum (2048)");
    return GBNUTS_USAGE;
  }
  // Row splits exactly as the regular entry point chooses them.
  int S = choose_splits(desc, C, precision);
  constexpr int kMaxSplits = 512;
  if (S > kMaxSplits) S = kMaxSplits;
  const int NP = n_partials(desc);
  const size_t partial_bytes = align256((size_t)S * C * NP * sizeof(double));
  const size_t gz_bytes = desc.off_z >= 0 ? align256((size_t)C * desc.J * sizeof(double)) : 0;
  const size_t split_bytes = align256((size_t)(S + 1) * sizeof(long long));
  const size_t need = partial_bytes + gz_bytes + split_bytes + 256;
  if (need > kNoAllocScratchBytes) {
    set_last_error("the request needs " + std::to_string(need) +
                   " bytes of scratch; the no-allocation entry point has " +
                   std::to_string(kNoAllocScratchBytes) + " (use fewer chains per call)");
    return GBNUTS_USAGE;
  }
  void* base = nullptr;
  rc = scratch_address(&base);
  if (rc) return rc;
  unsigned char* b = static_cast<unsigned char*>(base);
  GradWorkspace ws;
  ws.C = C;
  ws.S = S;
  ws.NP = NP;
  ws.precision = precision;
  ws.partial = reinterpret_cast<double*>(b);
  ws.gz = desc.off_z >= 0 ? reinterpret_cast<double*>(b + partial_bytes) : nullptr;
  ws.split_rows = reinterpret_cast<long long*>(b + partial_bytes + gz_bytes);
  ws.err = reinterpret_cast<int*>(b + partial_bytes + gz_bytes + split_bytes);
  (void)group_off;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  noalloc_setup_kernel<<<1, 256, 0, st>>>(desc.N, S, desc.J,
                                          desc.off_z >= 0 ? desc.group : nullptr,
                                          ws.split_rows, ws.err);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error(std::string("scratch set-up: ") + cudaGetErrorString(e));
    return GBNUTS_SOFTWARE;
  }
  // The group sums are cleared by the launch itself; the partials are fully
  // overwritten for every active chain.
  return launch_log_prob_grad(desc, precision, d_theta, desc.D, C, nullptr, d_lp, d_grad,
                              desc.D, 1, 1, ws, st, nullptr, nullptr);
}
