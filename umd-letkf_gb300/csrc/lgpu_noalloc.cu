// lgpu_noalloc.cu -- lgpu_get_obslist_noalloc: the local-observation-list
// query of lgpu_get_obslist for callers that must not allocate memory.
//
// Who needs it: hosts that run the analysis inside a memory manager of their
// own -- a model that takes its device memory as one pool at start-up and
// hands it out itself, or a real-time cycling driver whose memory footprint
// is fixed once it starts.  lgpu_get_obslist grows a device buffer the first
// time a list is larger than the last one, which such hosts do not allow.
// This variant never calls cudaMalloc or cudaFree: its scratch lives in one
// file-scope __device__ array of fixed size, so its memory cost is paid
// once, when the library is loaded onto a device, and stays resident on
// every device that loads the library until the process exits.
//
// Limits and contract:
//   - at most LGPU_NOALLOC_MAX_LIST observations in the handle's table (the
//     worst case of one list); larger tables are rejected with
//     LGPU_ERR_CAPACITY before any work is launched;
//   - all calls share the one scratch array, which keeps the contents of the
//     last call: the counters and the table-sized flag array are cleared on
//     every call before the kernels run; calls whose work overlaps on the GPU
//     (concurrent calls on several handles/threads of one device) race on
//     that array and must be serialised by the caller;
//   - the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress, with that device current).
#include <mutex>
#include <cstdio>

#include "lgpu_internal.cuh"

namespace lgpu {
cudaError_t launch_obslist_noalloc(cudaStream_t st, int gid, const ColPar *cp_col, const DevLoc &loc, ObsSorted obs,
                                   const IndexGeom *geom, int nobs, int *scratch);
}

namespace {

constexpr int kMaxList = LGPU_NOALLOC_MAX_LIST;
// layout (ints): [0..64) counters (two used), then one slot per observation
// of the table: kept flag, weight; then the list in canonical order: index,
// weight
constexpr size_t kScratchInts = 64 + 4 * (size_t)kMaxList;

static __device__ __align__(256) int g_noalloc_scratch[kScratchInts];

std::mutex g_mu;
int *g_ptr[64] = {};   // device address of g_noalloc_scratch per device ordinal

}  // namespace

namespace lgpu {

namespace {

// search + localize of one (column, group): the kept observations are marked
// in the per-observation slots (flag and weight at the observation's index;
// each observation is met at most once), counters [0] kept, [1] candidates
__global__ void k_obslist_noalloc(int gid, const ColPar *cpp, DevLoc loc, ObsSorted obs, const IndexGeom *geom,
                                  int *scratch) {
  int *flag = scratch + 64;
  float *wr = reinterpret_cast<float *>(scratch + 64 + kMaxList);
  const ColPar cp = *cpp;
  list_search(gid, cp, loc, obs, geom, scratch, [&](int p, float r) {
    const int i = obs.idx[p];
    flag[i] = 1;
    wr[i] = r;
  });
}

// canonical order (ascending observation index): one block scans the flags
// of the nobs slots; thread t owns a contiguous range of slots, so the ranks
// come from an exclusive scan of the per-thread counts
constexpr int kOrderThreads = 1024;

__global__ void __launch_bounds__(kOrderThreads) k_order_noalloc(int *scratch, int nobs) {
  __shared__ int wsum[kOrderThreads / 32];
  const int *flag = scratch + 64;
  const float *wr = reinterpret_cast<const float *>(scratch + 64 + kMaxList);
  int *sidx = scratch + 64 + 2 * (size_t)kMaxList;
  float *sr = reinterpret_cast<float *>(scratch + 64 + 3 * (size_t)kMaxList);
  const int per = (nobs + kOrderThreads - 1) / kOrderThreads;
  const int lo = min(nobs, (int)threadIdx.x * per), hi = min(nobs, lo + per);
  int c = 0;
  for (int i = lo; i < hi; i++) c += flag[i];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = c;   // inclusive scan within the warp
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (w == 0) {   // inclusive scan of the warp totals
    int v = wsum[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += y;
    }
    wsum[lane] = v;
  }
  __syncthreads();
  int pos = x - c + (w > 0 ? wsum[w - 1] : 0);
  for (int i = lo; i < hi; i++)
    if (flag[i]) {
      sidx[pos] = i;
      sr[pos] = wr[i];
      pos++;
    }
}

}  // namespace

cudaError_t launch_obslist_noalloc(cudaStream_t st, int gid, const ColPar *cp_col, const DevLoc &loc, ObsSorted obs,
                                   const IndexGeom *geom, int nobs, int *scratch) {
  if (nobs < 0 || nobs > kMaxList) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(scratch, 0, (64 + (size_t)nobs) * sizeof(int), st);   // counters + flags
  if (e != cudaSuccess) return e;
  k_obslist_noalloc<<<1, 256, 0, st>>>(gid, cp_col, loc, obs, geom, scratch);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  k_order_noalloc<<<1, kOrderThreads, 0, st>>>(scratch, nobs);
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
