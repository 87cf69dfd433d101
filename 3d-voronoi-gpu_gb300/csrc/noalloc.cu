// Grid kNN for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: a host framework that
// owns the whole device memory pool and forbids allocations outside it, or a
// latency-critical loop where cudaMalloc's implicit synchronisation of the
// device is not acceptable.  vgb_knn_noalloc serves them: the caller passes
// device buffers for the points and the results, and every intermediate array
// of the grid kNN (points with ids, their grid-ordered copy, cell starts, the
// sort's keys, digit counts and scan tile sums, the id -> position map)
// lives in one file-scope static device array, sized for at most
// VGB_NOALLOC_MAX_POINTS points.  Every GPU that loads this library holds that
// array (about 2.9 MB) until the process exits.
//
// Host code never dereferences the array's name: on the host it is only a
// stand-in, not a device address.  The first call on each device (with that
// device current) looks the array's device address up with
// cudaGetSymbolAddress and records the kNN kernel's resident block count for
// that device (an occupancy query); later calls on the device reuse both.
// That first call should therefore come before any stream capture.  Every
// call shares the one array and leaves its contents behind (each call clears
// the counters it needs), so calls that overlap on the GPU -- two streams, or
// two host threads on one device -- race on it.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/voronoi_gb300.h"
#include "vgb_common.cuh"

namespace vgb {
namespace {

constexpr int NA_MAX_POINTS = VGB_NOALLOC_MAX_POINTS;
constexpr int NA_MAX_DIM = 32;  // vgb_grid_dim(65536) is 28
constexpr long long NA_MAX_CELLS = (long long)NA_MAX_DIM * NA_MAX_DIM * NA_MAX_DIM;

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// byte offsets of the scratch arrays
constexpr size_t OFF_IN = 0;
constexpr size_t OFF_SORTED = OFF_IN + align256(sizeof(float4) * NA_MAX_POINTS);
constexpr size_t OFF_POS_OF_ID = OFF_SORTED + align256(sizeof(float4) * NA_MAX_POINTS);
constexpr size_t OFF_CELL_START = OFF_POS_OF_ID + align256(sizeof(int) * NA_MAX_POINTS);
constexpr size_t OFF_WORK = OFF_CELL_START + align256(sizeof(int) * (NA_MAX_CELLS + 1));
constexpr size_t SCRATCH_BYTES = OFF_WORK + align256(sizeof(int) * grid_sort_work_ints(NA_MAX_POINTS, NA_MAX_CELLS));

static __device__ __align__(256) unsigned char g_knn_scratch[SCRATCH_BYTES];

constexpr int NA_MAX_DEVICES = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch_ptr[NA_MAX_DEVICES] = {};

// Device address of the scratch array on the current device (set-up on the
// first call per device).
int scratch_for_current_device(unsigned char** out) {
  int dev = 0;
  VGB_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= NA_MAX_DEVICES) {
    set_error("vgb_knn_noalloc: device %d beyond the supported %d", dev, NA_MAX_DEVICES);
    return VGB_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    VGB_CUDA_TRY(cudaGetSymbolAddress(&p, g_knn_scratch));
    if (knn_prepare()) return VGB_ERR_CUDA;
    g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_ptr[dev];
  return VGB_OK;
}

__global__ void k_na_pack(const float* __restrict__ xyz, int n, float4* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], __int_as_float(i));
}

__global__ void k_na_perm(const float4* __restrict__ sorted, int n, unsigned* __restrict__ perm) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  perm[i] = (unsigned)__float_as_int(sorted[i].w);
}

}  // namespace
}  // namespace vgb

using namespace vgb;

extern "C" int vgb_knn_noalloc(const float* d_points, int n, int k, unsigned* d_knn, unsigned* d_perm,
                               void* stream) {
  if (!d_points || !d_knn || !d_perm) {
    set_error("vgb_knn_noalloc: NULL buffer");
    return VGB_ERR_INVALID;
  }
  if (n < 2 || n > NA_MAX_POINTS) {
    set_error("vgb_knn_noalloc: %d points; this entry point takes 2 to %d (use kn_prepare_ex for more)", n,
              NA_MAX_POINTS);
    return VGB_ERR_INVALID;
  }
  if (k < 1 || k > MAX_SITE_K || k >= n) {
    set_error("vgb_knn_noalloc: k=%d must be in [1, min(%d, n-1)]", k, MAX_SITE_K);
    return VGB_ERR_INVALID;
  }
  const int dim = vgb_grid_dim(n);
  if (dim > NA_MAX_DIM) {
    set_error("vgb_knn_noalloc: grid side %d above %d", dim, NA_MAX_DIM);
    return VGB_ERR_INVALID;
  }
  unsigned char* base = nullptr;
  int rc = scratch_for_current_device(&base);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  float4* in = reinterpret_cast<float4*>(base + OFF_IN);
  float4* sorted = reinterpret_cast<float4*>(base + OFF_SORTED);
  int* pos_of_id = reinterpret_cast<int*>(base + OFF_POS_OF_ID);
  int* cell_start = reinterpret_cast<int*>(base + OFF_CELL_START);
  int* work = reinterpret_cast<int*>(base + OFF_WORK);
  k_na_pack<<<(n + 255) / 256, 256, 0, st>>>(d_points, n, in);
  VGB_CUDA_TRY(cudaGetLastError());
  // grid_sort clears the cell counters and fill counters it needs at zero
  const ProbDesc lone = lone_problem(n, dim, 0, k);
  if (grid_sort(in, sorted, n, (long long)dim * dim * dim, nullptr, nullptr, lone, cell_start, work, st))
    return VGB_ERR_CUDA;
  if (knn_sites(sorted, n, cell_start, nullptr, nullptr, lone, k, pos_of_id, d_knn, nullptr, st)) return VGB_ERR_CUDA;
  k_na_perm<<<(n + 255) / 256, 256, 0, st>>>(sorted, n, d_perm);
  VGB_CUDA_TRY(cudaGetLastError());
  return VGB_OK;
}
