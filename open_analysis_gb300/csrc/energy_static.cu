// Field energy without any device allocation.
//
// Some callers cannot allocate device memory: a plugin whose host application owns every device
// allocation (it hands the library only buffers it made itself and counts every byte), and
// services that reserve their device memory at start-up and must not grow it afterwards. This
// entry point computes the same energy as oafdtd_energy from field arrays the caller already holds
// on the device, with its per-plane partial sums in a file-scope device array instead of a
// cudaMalloc'd buffer.
//
// Limits and sharing:
//  * the scratch holds kMaxPartials doubles (512 KiB) on every GPU that loads the library, for
//    the life of the process; a problem needs 6 * batch * (nz + 2) partials and is rejected with
//    OAFDTD_E_INVALID beyond that;
//  * every call in the process shares the one array, whatever stream it is given: calls that
//    overlap on the GPU (different streams or threads) race and must be serialised by the caller.
//    Each call writes every partial it later reads, so nothing needs clearing between calls;
//  * the call is synchronous: it copies the six component sums to the host and synchronises the
//    caller's stream before it returns. It therefore cannot run on a stream that is being captured
//    (or on the legacy default stream while another stream captures in global mode); it checks
//    and returns OAFDTD_E_INVALID there, before it launches anything;
//  * the first call in a device's context looks the array's device address up
//    (cudaGetSymbolAddress, with that device current) and caches it, keyed by the context's
//    unique id, so a context that was reset and created again looks it up anew. That first
//    lookup may load the library's module on the device (with lazy loading), which the driver
//    backs with memory for the module's code and this array.
#include <mutex>
#include <string>

#include "../../include/oafdtd.h"
#include "oafdtd_internal.cuh"

constexpr int kMaxPartials = 65536;

// The scratch: kMaxPartials partial sums and the six component sums after them.
static __device__ __align__(256) double g_energy_scratch[kMaxPartials + 8];

namespace {

constexpr int kMaxDevices = 256;
constexpr double kEps0 = 1.0 / (4e-7 * 3.14159265358979323846 * 299792458.0 * 299792458.0);
constexpr double kMu0 = 4e-7 * 3.14159265358979323846;

std::mutex g_scratch_mu;
struct ScratchSlot {
  unsigned long long ctx_id;  // unique id of the context the address belongs to (0: none)
  double* ptr;
};
ScratchSlot g_scratch[kMaxDevices] = {};

// Driver entry points for the current context and its process-unique id (CUDA 12.0 and later).
using CtxGetCurrent = CUresult (*)(CUcontext*);
using CtxGetId = CUresult (*)(CUcontext, unsigned long long*);

template <typename F>
F driver_entry(const char* name) {
  void* p = nullptr;
  cudaDriverEntryPointQueryResult q{};
  if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess)
    return nullptr;
  return reinterpret_cast<F>(p);
}

// Id of the context current on this thread; 0 when none is current or the driver cannot say.
unsigned long long current_context_id() {
  static const CtxGetCurrent get_current = driver_entry<CtxGetCurrent>("cuCtxGetCurrent");
  static const CtxGetId get_id = driver_entry<CtxGetId>("cuCtxGetId");
  if (get_current == nullptr || get_id == nullptr) return 0;
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// One block per (component, batch member, z plane): weighted sum of the plane, fixed order.
template <typename real>
__global__ void __launch_bounds__(256) plane_energy_kernel(oafdtd_energy_view v, double* partial) {
  __shared__ double warp_sum[8];
  const int cc = blockIdx.y;  // 0..2 E, 3..5 H
  const int X = v.pitch, Y = v.ny + 2, Z = v.nz + 2;
  const int plane = blockIdx.x;  // b * Z + k
  const int k = plane % Z;
  const real* F = static_cast<const real*>(v.field[cc]) + (long long)plane * Y * X;
  const int c = cc % 3;
  const bool is_e = cc < 3;
  const double* wx = (is_e ? (c != 0) : (c == 0)) ? v.node_w[0] : v.cell_w[0];
  const double* wy = (is_e ? (c != 1) : (c == 1)) ? v.node_w[1] : v.cell_w[1];
  const double* wz = (is_e ? (c != 2) : (c == 2)) ? v.node_w[2] : v.cell_w[2];
  const uint16_t* idx = is_e ? v.idx[c] + (long long)k * Y * X : nullptr;
  double acc = 0.0;
  for (int j = 0; j < Y; ++j) {
    const double wyz = wy[j] * wz[k];
    for (int i = threadIdx.x; i < X; i += blockDim.x) {
      const double f = (double)F[(long long)j * X + i];
      double term = wx[i] * wyz * f * f;
      if (is_e) term *= v.eps_tab[idx[(long long)j * X + i]] * kEps0;
      acc += term;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < 8; ++w) s += warp_sum[w];
    partial[(long long)cc * gridDim.x + plane] = s;
  }
}

__global__ void plane_energy_sum_kernel(const double* partial, int per_comp, double* sums) {
  const int cc = threadIdx.x;
  if (cc >= 6) return;
  double s = 0.0;
  for (int q = 0; q < per_comp; ++q) s += partial[(long long)cc * per_comp + q];
  sums[cc] = s;
}

int fail_static(int code, const std::string& msg) {
  oafdtd::set_last_error(msg);
  return code;
}

// Device address of the scratch array in the current device's context, looked up once per
// context (and on every call where the driver cannot name the context).
int scratch_address(double** out) {
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return fail_static(OAFDTD_E_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(err));
  if (dev < 0 || dev >= kMaxDevices) return fail_static(OAFDTD_E_NODEVICE, "device index beyond the scratch table");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  const unsigned long long id = current_context_id();
  ScratchSlot& slot = g_scratch[dev];
  if (id == 0 || slot.ctx_id != id || slot.ptr == nullptr) {
    void* p = nullptr;
    err = cudaGetSymbolAddress(&p, g_energy_scratch);
    if (err != cudaSuccess)
      return fail_static(OAFDTD_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(err));
    slot.ptr = static_cast<double*>(p);
    slot.ctx_id = current_context_id();  // the lookup made the context current if it was not
  }
  *out = slot.ptr;
  return OAFDTD_OK;
}

}  // namespace

extern "C" int oafdtd_energy_noalloc(const oafdtd_energy_view* view, double* out) {
  if (view == nullptr || out == nullptr) return fail_static(OAFDTD_E_INVALID, "null argument");
  const oafdtd_energy_view& v = *view;
  if (v.real_bytes != 4 && v.real_bytes != 8) return fail_static(OAFDTD_E_INVALID, "real_bytes must be 4 or 8");
  if (v.nx < 1 || v.ny < 1 || v.nz < 1 || v.batch < 1 || v.pitch < v.nx + 2 || v.pitch % 32 != 0)
    return fail_static(OAFDTD_E_INVALID, "bad grid or batch size");
  for (int c = 0; c < 6; ++c)
    if (v.field[c] == nullptr) return fail_static(OAFDTD_E_INVALID, "null field pointer");
  for (int a = 0; a < 3; ++a)
    if (v.idx[a] == nullptr || v.node_w[a] == nullptr || v.cell_w[a] == nullptr)
      return fail_static(OAFDTD_E_INVALID, "null index or weight pointer");
  if (v.eps_tab == nullptr) return fail_static(OAFDTD_E_INVALID, "null eps_tab pointer");
  const long long per_comp = (long long)v.batch * (v.nz + 2);
  if (6 * per_comp > kMaxPartials)
    return fail_static(OAFDTD_E_INVALID, "6 * batch * (nz + 2) = " + std::to_string(6 * per_comp) +
                                             " partial sums exceed the static scratch of " +
                                             std::to_string(kMaxPartials));
  cudaStream_t s = static_cast<cudaStream_t>(v.stream);
  // the call ends in a read-back and a synchronise, which a stream capture cannot hold
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaError_t err = cudaStreamIsCapturing(s, &cap);
  if (err != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
    if (err != cudaSuccess) cudaGetLastError();  // the query's error is not sticky: clear it
    return fail_static(OAFDTD_E_INVALID,
                       "oafdtd_energy_noalloc is synchronous and cannot run while its stream (or, for the legacy "
                       "default stream, any stream in global mode) is being captured");
  }
  double* scratch = nullptr;
  if (int rc = scratch_address(&scratch)) return rc;
  dim3 grid((unsigned)per_comp, 6);
  if (v.real_bytes == 4)
    plane_energy_kernel<float><<<grid, 256, 0, s>>>(v, scratch);
  else
    plane_energy_kernel<double><<<grid, 256, 0, s>>>(v, scratch);
  err = cudaGetLastError();
  if (err != cudaSuccess) return fail_static(OAFDTD_E_CUDA, std::string("energy kernel: ") + cudaGetErrorString(err));
  double* sums = scratch + kMaxPartials;
  plane_energy_sum_kernel<<<1, 32, 0, s>>>(scratch, (int)per_comp, sums);
  err = cudaGetLastError();
  if (err != cudaSuccess) return fail_static(OAFDTD_E_CUDA, std::string("energy sum: ") + cudaGetErrorString(err));
  double parts[6];
  err = cudaMemcpyAsync(parts, sums, sizeof(parts), cudaMemcpyDeviceToHost, s);
  if (err == cudaSuccess) err = cudaStreamSynchronize(s);
  if (err != cudaSuccess) return fail_static(OAFDTD_E_CUDA, std::string("energy read-back: ") + cudaGetErrorString(err));
  double total = 0.0;
  for (int c = 0; c < 3; ++c) {
    total += 0.5 * parts[c];
    total += 0.5 * kMu0 * parts[3 + c];
  }
  *out = total;
  return OAFDTD_OK;
}
