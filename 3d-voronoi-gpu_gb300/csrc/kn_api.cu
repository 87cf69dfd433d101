// kn_* drop-in (include/knearests.h) over the grid sort and kNN kernels.
// Replaces kn_prepare / kn_solve / kn_free / kn_print_stats / kn_get_*
// (knearests.cu:149-460).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <vector>

#include "../../include/knearests.h"
#include "../../include/voronoi_gb300.h"
#include "vgb_common.cuh"

using namespace vgb;

namespace {

struct KnImpl {
  float4* in = nullptr;      // input points with ids
  float4* sorted = nullptr;  // grid order with ids
  int* cell_start = nullptr;
  int* cell_fill = nullptr;
  int* grid_work = nullptr;  // grid_sort_work_ints(n, cells)
  int* scan_tmp = nullptr;
  int* pos_of_id = nullptr;
};

__global__ void k_kn_pack(const float* __restrict__ xyz, int n, float4* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], __int_as_float(i));
}

// Reference-layout views of the sorted grid: float3 points, permutation,
// per-cell counts and starts.
__global__ void k_kn_views(const float4* __restrict__ sorted, int n, float3* __restrict__ pts,
                           unsigned* __restrict__ perm) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 p = sorted[i];
  pts[i] = make_float3(p.x, p.y, p.z);
  perm[i] = (unsigned)__float_as_int(p.w);
}

__global__ void k_kn_cells(const int* __restrict__ start, int ncell, int* __restrict__ counters,
                           int* __restrict__ ptrs) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  ptrs[c] = start[c];
  counters[c] = start[c + 1] - start[c];
}

void kn_release(kn_problem* kn) {
  if (!kn) return;
  KnImpl* im = static_cast<KnImpl*>(kn->impl);
  if (im) {
    void* b[] = {im->in, im->sorted, im->cell_start, im->cell_fill, im->grid_work, im->scan_tmp, im->pos_of_id};
    for (void* p : b)
      if (p) cudaFree(p);
    delete im;
  }
  void* b[] = {kn->d_permutation, kn->d_counters, kn->d_ptrs, kn->d_globcounter, kn->d_stored_points,
               kn->d_knearests};
  for (void* p : b)
    if (p) cudaFree(p);
  free(kn);
}

[[noreturn]] void kn_fail(const char* where) {
  fprintf(stderr, "Failed (%s): %s\n", where, vgb_last_error());
  exit(EXIT_FAILURE);
}

}  // namespace

extern "C" {

int kn_prepare_ex(kn_problem** out, const float* xyz, int n, int k) {
  if (!out || !xyz || n <= 1 || k < 1 || k > MAX_SITE_K || k >= n) {
    set_error("kn_prepare: need 1 <= k <= %d and k < numpoints (k=%d, n=%d)", MAX_SITE_K, k, n);
    return VGB_ERR_INVALID;
  }
  *out = nullptr;
  kn_problem* kn = (kn_problem*)calloc(1, sizeof(kn_problem));
  KnImpl* im = new KnImpl();
  if (!kn || !im) { set_error("host allocation failed"); free(kn); delete im; return VGB_ERR_NOMEM; }
  kn->impl = im;
  kn->allocated_points = n;
  kn->k = k;
  int dim = vgb_grid_dim(n);
  kn->dimx = kn->dimy = kn->dimz = dim;
  long long nc = (long long)dim * dim * dim;
  auto A = [&](void** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 1);
    if (e != cudaSuccess) { set_error("cudaMalloc: %s", cudaGetErrorString(e)); return false; }
    return true;
  };
  bool ok = A((void**)&im->in, sizeof(float4) * n) && A((void**)&im->sorted, sizeof(float4) * n) &&
            A((void**)&im->cell_start, sizeof(int) * (nc + 1)) && A((void**)&im->cell_fill, sizeof(int) * nc) &&
            A((void**)&im->grid_work, sizeof(int) * grid_sort_work_ints(n, nc)) &&
            A((void**)&im->scan_tmp, sizeof(int) * scan_tmp_ints(nc + 1)) &&
            A((void**)&im->pos_of_id, sizeof(int) * n) &&
            A((void**)&kn->d_permutation, sizeof(unsigned) * n) && A((void**)&kn->d_counters, sizeof(int) * nc) &&
            A((void**)&kn->d_ptrs, sizeof(int) * nc) && A((void**)&kn->d_globcounter, sizeof(int)) &&
            A((void**)&kn->d_stored_points, sizeof(float3) * n) &&
            A((void**)&kn->d_knearests, sizeof(unsigned) * (size_t)n * k);
  if (!ok) { kn_release(kn); return VGB_ERR_NOMEM; }
  float* stage = nullptr;
  if (!A((void**)&stage, sizeof(float) * 3 * n)) { kn_release(kn); return VGB_ERR_NOMEM; }
  cudaStream_t st = 0;
  cudaError_t ce = cudaMemcpy(stage, xyz, sizeof(float) * 3 * n, cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) {
    k_kn_pack<<<(n + 255) / 256, 256, 0, st>>>(stage, n, im->in);
    ce = cudaGetLastError();
  }
  if (ce != cudaSuccess) { set_error("kn_prepare upload: %s", cudaGetErrorString(ce)); cudaFree(stage); kn_release(kn); return VGB_ERR_CUDA; }
  const ProbDesc lone = lone_problem(n, dim, 0, k);
  int rc = grid_sort(im->in, im->sorted, n, nc, nullptr, nullptr, lone, im->cell_start, im->grid_work, st);
  if (!rc) {
    k_kn_views<<<(n + 255) / 256, 256, 0, st>>>(im->sorted, n, kn->d_stored_points, kn->d_permutation);
    k_kn_cells<<<(unsigned)((nc + 255) / 256), 256, 0, st>>>(im->cell_start, (int)nc, kn->d_counters, kn->d_ptrs);
    ce = cudaMemcpyAsync(kn->d_globcounter, im->cell_start + nc, sizeof(int), cudaMemcpyDeviceToDevice, st);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(kn->d_knearests, 0xff, sizeof(unsigned) * (size_t)n * k, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) { set_error("kn_prepare: %s", cudaGetErrorString(ce)); rc = VGB_ERR_CUDA; }
  }
  cudaFree(stage);
  if (rc) { kn_release(kn); return rc; }
  *out = kn;
  return VGB_OK;
}

int kn_solve_ex(kn_problem* kn) {
  if (!kn || !kn->impl) { set_error("kn_solve: NULL problem"); return VGB_ERR_INVALID; }
  KnImpl* im = static_cast<KnImpl*>(kn->impl);
  if (knn_prepare()) return VGB_ERR_CUDA;
  const ProbDesc lone = lone_problem(kn->allocated_points, kn->dimx, 0, kn->k);
  if (knn_sites(im->sorted, kn->allocated_points, im->cell_start, nullptr, nullptr, lone, kn->k, im->pos_of_id,
                kn->d_knearests, nullptr, 0))
    return VGB_ERR_CUDA;
  VGB_CUDA_TRY(cudaStreamSynchronize(0));
  return VGB_OK;
}

int kn_free_ex(kn_problem* kn) {
  kn_release(kn);
  return VGB_OK;
}

kn_problem* kn_prepare_k(const float3* points, int numpoints, int k) {
  kn_problem* kn = nullptr;
  if (kn_prepare_ex(&kn, reinterpret_cast<const float*>(points), numpoints, k) != VGB_OK) kn_fail("kn_prepare");
  return kn;
}

kn_problem* kn_prepare(float3* points, int numpoints) { return kn_prepare_k(points, numpoints, 90); }

void kn_solve(kn_problem* kn) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a);
  if (kn_solve_ex(kn) != VGB_OK) kn_fail("kn_solve");
  cudaEventRecord(b);
  cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  fprintf(stderr, "kn_solve: %g msec\n", ms);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
}

void kn_free(kn_problem** kn) {
  if (!kn) return;
  kn_release(*kn);
  *kn = nullptr;
}

static void* kn_copy(const void* dev, size_t bytes, const char* what) {
  void* h = malloc(bytes ? bytes : 1);
  cudaError_t e = h ? cudaMemcpy(h, dev, bytes, cudaMemcpyDeviceToHost) : cudaErrorMemoryAllocation;
  if (e != cudaSuccess) {
    fprintf(stderr, "[%s] Failed to copy from device to host (error code %s)!\n", what, cudaGetErrorString(e));
    exit(EXIT_FAILURE);
  }
  return h;
}

float3* kn_get_points(kn_problem* kn) {
  return (float3*)kn_copy(kn->d_stored_points, sizeof(float3) * kn->allocated_points, "kn_get_points");
}

unsigned int* kn_get_knearests(kn_problem* kn) {
  return (unsigned*)kn_copy(kn->d_knearests, sizeof(unsigned) * (size_t)kn->allocated_points * kn->k,
                            "kn_get_knearests");
}

unsigned int* kn_get_permutation(kn_problem* kn) {
  return (unsigned*)kn_copy(kn->d_permutation, sizeof(unsigned) * kn->allocated_points, "kn_get_permutation");
}

// Points-per-cell histogram (knearests.cu:434-460).
void kn_print_stats(kn_problem* kn) {
  long long nc = (long long)kn->dimx * kn->dimy * kn->dimz;
  int* c = (int*)kn_copy(kn->d_counters, sizeof(int) * nc, "kn_print_stats");
  long long tot = 0;
  int cmin = 1 << 30, cmax = 0;
  std::map<int, int> histo;
  for (long long i = 0; i < nc; ++i) {
    histo[c[i]]++;
    cmin = c[i] < cmin ? c[i] : cmin;
    cmax = c[i] > cmax ? c[i] : cmax;
    tot += c[i];
  }
  fprintf(stderr, "Grid:  points per cell: %d (min), %d (max), %g avg, total %lld\n", cmin, cmax,
          kn->allocated_points / (double)nc, tot);
  for (auto& h : histo) fprintf(stderr, "[%d] => %d\n", h.first, h.second);
  free(c);
}

}  // extern "C"
