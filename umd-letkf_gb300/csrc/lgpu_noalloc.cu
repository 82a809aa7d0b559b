// lgpu_noalloc.cu -- lgpu_get_obslist_noalloc: the local-observation-list
// query of lgpu_get_obslist for callers that must not allocate memory.
//
// Who needs it: hosts that run the analysis inside a memory manager of their
// own (a model's pre-allocated device pool, a real-time cycling driver that
// forbids allocation after start-up, code running while a CUDA stream is
// being captured).  lgpu_get_obslist grows a device buffer the first time a
// list is larger than the last one; this variant never calls cudaMalloc or
// cudaFree: its scratch lives in one file-scope __device__ array of fixed
// size, so its memory cost is paid once, when the library is loaded onto a
// device, and stays resident on every device that loads the library until
// the process exits.
//
// Limits and contract:
//   - at most LGPU_NOALLOC_MAX_LIST observations in the handle's table (the
//     worst case of one list); larger tables are rejected with
//     LGPU_ERR_CAPACITY before any work is launched;
//   - all calls share the one scratch array, which keeps the contents of the
//     last call: the two counters are cleared on every call before the
//     kernels run; calls whose work overlaps on the GPU (concurrent calls on
//     several handles/threads of one device) race on that array and must be
//     serialised by the caller;
//   - the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress, with that device current); make that first call
//     before any stream capture.
#include <mutex>
#include <cstdio>

#include "lgpu_internal.cuh"

namespace lgpu {
cudaError_t launch_obslist_noalloc(cudaStream_t st, int gid, const ColPar *cp_col, const DevLoc &loc, ObsSorted obs,
                                   const IndexGeom *geom, int nmax, int *scratch);
}

namespace {

constexpr int kMaxList = LGPU_NOALLOC_MAX_LIST;
// layout (ints): [0..64) counters (two used), then raw idx, raw r, sorted idx, sorted r
constexpr size_t kScratchInts = 64 + 4 * (size_t)kMaxList;

static __device__ __align__(256) int g_noalloc_scratch[kScratchInts];

std::mutex g_mu;
int *g_ptr[64] = {};   // device address of g_noalloc_scratch per device ordinal

}  // namespace

namespace lgpu {

namespace {

// search + localize of one (column, group) into the fixed scratch: entries in
// cell order, counters [0] kept, [1] candidates
__global__ void k_obslist_noalloc(int gid, const ColPar *cpp, DevLoc loc, ObsSorted obs, const IndexGeom *geom,
                                  int *scratch) {
  int *counts = scratch;
  int *ridx = scratch + 64;
  float *rr = reinterpret_cast<float *>(scratch + 64 + kMaxList);
  const ColPar cp = *cpp;
  const float hq = fminf(cp.rmax / 12742000.0f, 1.5707963f);
  const float sh = sinf(hq);
  const float c2max = 4.0f * sh * sh * 1.0001f + 1e-12f;
  for (int b = cp.b0; b <= cp.b1; b++) {
    const int nl = geom->nlon[b], off = geom->off[b];
    int runs[2][2] = {{0, 0}, {0, 0}};
    bool whole = cp.dlon >= 180.0f;
    int clo = 0, chi = nl - 1;
    if (!whole) {
      clo = (int)floorf((cp.lonn - cp.dlon) * (float)nl / 360.0f);
      chi = (int)floorf((cp.lonn + cp.dlon) * (float)nl / 360.0f);
      if (chi - clo + 1 >= nl) whole = true;
    }
    if (whole) { runs[0][0] = obs.cell_start[off]; runs[0][1] = obs.cell_start[off + nl]; }
    else if (clo < 0) {
      runs[0][0] = obs.cell_start[off + clo + nl]; runs[0][1] = obs.cell_start[off + nl];
      runs[1][0] = obs.cell_start[off]; runs[1][1] = obs.cell_start[off + chi + 1];
    } else if (chi >= nl) {
      runs[0][0] = obs.cell_start[off + clo]; runs[0][1] = obs.cell_start[off + nl];
      runs[1][0] = obs.cell_start[off]; runs[1][1] = obs.cell_start[off + chi - nl + 1];
    } else { runs[0][0] = obs.cell_start[off + clo]; runs[0][1] = obs.cell_start[off + chi + 1]; }
    for (int q = 0; q < 2; q++)
      for (int p = runs[q][0] + threadIdx.x; p < runs[q][1]; p += blockDim.x) {
        const float4 A = obs.A[p];
        const float c2 = chord2_exact(cp.ux, cp.uy, cp.uz, A.x, A.y, A.z);
        if (c2 > c2max) continue;
        const float d = dist_from_chord2(c2);
        if (d > cp.rmax) continue;
        atomicAdd(&counts[1], 1);
        const float4 B = obs.B[p];
        const float r = localize(loc, cp, gid, d, B.y, B.z, B.w);
        if (r > kKeep) {
          const int s = atomicAdd(&counts[0], 1);
          if (s < kMaxList) { ridx[s] = obs.idx[p]; rr[s] = r; }
        }
      }
  }
}

// canonical order (ascending observation index; indices are unique)
__global__ void k_rank_noalloc(int *scratch) {
  const int n = min(scratch[0], kMaxList);
  const int *ridx = scratch + 64;
  const float *rr = reinterpret_cast<const float *>(scratch + 64 + kMaxList);
  int *sidx = scratch + 64 + 2 * (size_t)kMaxList;
  float *sr = reinterpret_cast<float *>(scratch + 64 + 3 * (size_t)kMaxList);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int v = ridx[t];
    int rank = 0;
    for (int j = 0; j < n; j++) rank += (ridx[j] < v);
    sidx[rank] = v;
    sr[rank] = rr[t];
  }
}

}  // namespace

cudaError_t launch_obslist_noalloc(cudaStream_t st, int gid, const ColPar *cp_col, const DevLoc &loc, ObsSorted obs,
                                   const IndexGeom *geom, int nmax, int *scratch) {
  (void)nmax;
  cudaError_t e = cudaMemsetAsync(scratch, 0, 64 * sizeof(int), st);
  if (e != cudaSuccess) return e;
  k_obslist_noalloc<<<1, 256, 0, st>>>(gid, cp_col, loc, obs, geom, scratch);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  k_rank_noalloc<<<64, 256, 0, st>>>(scratch);
  return cudaGetLastError();
}

// Device address of the scratch array on `device` (the caller has made it
// current).  Looked up once per device.
cudaError_t noalloc_scratch(int device, int **out) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
  if (!g_ptr[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_ptr[device] = static_cast<int *>(p);
  }
  *out = g_ptr[device];
  return cudaSuccess;
}

int noalloc_max_list() { return kMaxList; }

}  // namespace lgpu
