// otfem_pattern.cu -- builds on the GPU, once per mesh:
//  * the node -> (tet, slot) incidence lists in ascending tet order (the
//    per-node tet list of t4mesh_t4node.h:36, sorted);
//  * the K_row sparsity pattern: for every node i the ascending set of nodes j
//    that share a tet with i, which are exactly the keys that
//    p_i->K(p_j->idx()) creates in stiffness_assembly
//    (fem_stiffness_assembly.h:199-201; std::map keeps them sorted);
//  * for every pattern block the ascending-tet list of (tet, local i, local j)
//    contributions, used by the reference-order assembly gather.
// All steps are deterministic: counts by atomics, then per-node sorting.
#include <climits>

#include "otfem_internal.h"

namespace otfem {
namespace {

constexpr int kThreads = 256;
inline int blocks_for(long n) { long b = (n + kThreads - 1) / kThreads; return b > 0 ? int(b) : 1; }

__global__ void k_count_incidence(int T, const int4* __restrict__ tets, int* cnt) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  int4 n = tets[t];
  atomicAdd(cnt + n.x, 1);
  atomicAdd(cnt + n.y, 1);
  atomicAdd(cnt + n.z, 1);
  atomicAdd(cnt + n.w, 1);
}

// Exclusive scan of n ints into out[0..n] (out[n] = total), in three
// coalesced passes: each CTA scans a tile of 1024 (warp shuffles, then the
// warp totals), one CTA scans the tile totals, and every element gets its
// tile's offset.  Used only at set-up.
constexpr int kScanTile = 1024;

__global__ void k_scan_tiles(long n, const int* __restrict__ in, int* out, long* tile_sums) {
  __shared__ long warp_tot[kScanTile / 32];
  const long i = long(blockIdx.x) * kScanTile + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long v = i < n ? in[i] : 0;
  long x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    long w = lane < kScanTile / 32 ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kScanTile / 32) warp_tot[lane] = w;  // inclusive
  }
  __syncthreads();
  const long before = warp ? warp_tot[warp - 1] : 0;
  if (i < n) out[i] = int(before + x - v);
  if (threadIdx.x == kScanTile - 1) tile_sums[blockIdx.x] = before + x;
}

// In place: tile_sums[k] <- sum of tiles before k; out[n] = total.
__global__ void k_scan_tile_sums(long tiles, long* tile_sums, int* out, long n) {
  __shared__ long part[1024];
  const long chunk = (tiles + blockDim.x - 1) / blockDim.x;
  const long lo = threadIdx.x * chunk, hi = lo + chunk < tiles ? lo + chunk : tiles;
  long s = 0;
  for (long k = lo; k < hi; ++k) s += tile_sums[k];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    long acc = 0;
    for (int k = 0; k < int(blockDim.x); ++k) {
      const long v = part[k];
      part[k] = acc;
      acc += v;
    }
    out[n] = int(acc);
  }
  __syncthreads();
  long acc = part[threadIdx.x];
  for (long k = lo; k < hi; ++k) {
    const long v = tile_sums[k];
    tile_sums[k] = acc;
    acc += v;
  }
}

__global__ void k_scan_add(long n, const long* __restrict__ tile_sums, int* out) {
  const long i = long(blockIdx.x) * kScanTile + threadIdx.x;
  if (i < n) out[i] += int(tile_sums[blockIdx.x]);
}

cudaError_t scan_exclusive(Context& c, long n, const int* in, int* out) {
  const long tiles = (n + kScanTile - 1) / kScanTile;
  long* sums = nullptr;
  cudaError_t e = cudaMallocAsync(&sums, sizeof(long) * (tiles > 0 ? tiles : 1), c.stream);
  if (e != cudaSuccess) return e;
  if (tiles > 0) k_scan_tiles<<<unsigned(tiles), kScanTile, 0, c.stream>>>(n, in, out, sums);
  k_scan_tile_sums<<<1, 1024, 0, c.stream>>>(tiles, sums, out, n);
  if (tiles > 0) k_scan_add<<<unsigned(tiles), kScanTile, 0, c.stream>>>(n, sums, out);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  return cudaFreeAsync(sums, c.stream);
}

__global__ void k_fill_incidence(int T, const int4* __restrict__ tets, const int* __restrict__ ptr,
                                 int* cursor, int* ent) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  int4 n = tets[t];
  int nn[4] = {n.x, n.y, n.z, n.w};
  for (int s = 0; s < 4; ++s) {
    int pos = atomicAdd(cursor + nn[s], 1);
    ent[ptr[nn[s]] + pos] = t * 4 + s;
  }
}

__device__ void insertion_sort(int* a, int n) {
  for (int i = 1; i < n; ++i) {
    int v = a[i], j = i - 1;
    while (j >= 0 && a[j] > v) {
      a[j + 1] = a[j];
      --j;
    }
    a[j + 1] = v;
  }
}

// Warp-wide sorts of short lists: a warp sorts one list of up to kWarpSortMax
// ints in its shared-memory segment by a bitonic network (lists padded with
// INT_MAX to the next power of two, at least 32), each lane taking every
// 32nd compare-exchange of a step.  Longer lists (not met on block meshes,
// whose nodes touch at most 24 tets) fall back to lane 0's insertion sort.
constexpr int kWarpSortMax = 256;
constexpr int kSortWarps = 8;  // warps per CTA of the warp-sort kernels

__device__ void warp_bitonic_sort(int* s, int P) {
  const int lane = threadIdx.x & 31;
  for (int k = 2; k <= P; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < P; i += 32) {
        const int l = i ^ j;
        if (l > i) {
          const int a = s[i], b = s[l];
          const bool up = (i & k) == 0;
          if ((a > b) == up) {
            s[i] = b;
            s[l] = a;
          }
        }
      }
      __syncwarp();
    }
}

__device__ __forceinline__ int sort_size(int m) {
  int P = 32;
  while (P < m) P <<= 1;
  return P;
}

// Node i's incidence entries (tet << 2 | slot) in ascending order, in place.
__global__ void k_sort_incidence(int N, const int* __restrict__ ptr, int* ent) {
  __shared__ int seg[kSortWarps][kWarpSortMax];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int i = blockIdx.x * kSortWarps + w;
  if (i >= N) return;
  int* a = ent + ptr[i];
  const int m = ptr[i + 1] - ptr[i];
  if (m > kWarpSortMax) {
    if (lane == 0) insertion_sort(a, m);
    return;
  }
  int* s = seg[w];
  const int P = sort_size(m);
  for (int k = lane; k < P; k += 32) s[k] = k < m ? a[k] : INT_MAX;
  __syncwarp();
  warp_bitonic_sort(s, P);
  for (int k = lane; k < m; k += 32) a[k] = s[k];
}

// Candidate neighbours of node i (the 4 nodes of each incident tet) sorted and
// de-duplicated in place in scratch[4*ptr[i] ...]; cnt[i] = distinct count.
// One warp per node: the node ids of its incident tets gathered into the
// warp's shared-memory segment, sorted (warp_bitonic_sort), and the distinct
// ids compacted by ballots into scratch[4*ptr[i] ...] in ascending order.
__global__ void k_row_unique(int N, const int4* __restrict__ tets, const int* __restrict__ ptr,
                             const int* __restrict__ ent, int* scratch, int* cnt) {
  __shared__ int seg[kSortWarps][kWarpSortMax];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int i = blockIdx.x * kSortWarps + w;
  if (i >= N) return;
  int* out = scratch + 4L * ptr[i];
  const int q0 = ptr[i], deg = ptr[i + 1] - q0, m = 4 * deg;
  if (m > kWarpSortMax) {
    if (lane == 0) {
      int k = 0;
      for (int q = q0; q < q0 + deg; ++q) {
        const int4 n = tets[ent[q] >> 2];
        out[k++] = n.x;
        out[k++] = n.y;
        out[k++] = n.z;
        out[k++] = n.w;
      }
      insertion_sort(out, m);
      int u = 0;
      for (int k2 = 0; k2 < m; ++k2)
        if (k2 == 0 || out[k2] != out[k2 - 1]) out[u++] = out[k2];
      cnt[i] = u;
    }
    return;
  }
  int* s = seg[w];
  const int P = sort_size(m);
  for (int q = lane; q < deg; q += 32) {
    const int4 n = tets[ent[q0 + q] >> 2];
    s[4 * q] = n.x;
    s[4 * q + 1] = n.y;
    s[4 * q + 2] = n.z;
    s[4 * q + 3] = n.w;
  }
  for (int k = m + lane; k < P; k += 32) s[k] = INT_MAX;
  __syncwarp();
  warp_bitonic_sort(s, P);
  int u = 0;
  for (int base = 0; base < m; base += 32) {
    const int k = base + lane;
    const bool first = k < m && (k == 0 || s[k] != s[k - 1]);
    const unsigned mask = __ballot_sync(0xffffffffu, first);
    if (first) out[u + __popc(mask & ((1u << lane) - 1u))] = s[k];
    u += __popc(mask);
  }
  if (lane == 0) cnt[i] = u;
}

__global__ void k_row_fill(int N, const int* __restrict__ ptr, const int* __restrict__ scratch,
                           const int* __restrict__ row_ptr, int* cols) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int* s = scratch + 4L * ptr[i];
  for (int k = row_ptr[i]; k < row_ptr[i + 1]; ++k) cols[k] = s[k - row_ptr[i]];
}

__device__ int find_col(const int* cols, int lo, int hi, int j) {
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (cols[mid] < j) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Per row: walk incident tets in ascending order; every local pair (li, lj)
// with tet[li] == i contributes once to block (i, tet[lj]).
__global__ void k_bc_count(int N, const int4* __restrict__ tets, const int* __restrict__ ptr,
                           const int* __restrict__ ent, const int* __restrict__ row_ptr,
                           const int* __restrict__ cols, int* bc_cnt) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  for (int q = ptr[i]; q < ptr[i + 1]; ++q) {
    int4 n4 = tets[ent[q] >> 2];
    int nn[4] = {n4.x, n4.y, n4.z, n4.w};
    for (int lj = 0; lj < 4; ++lj) bc_cnt[find_col(cols, row_ptr[i], row_ptr[i + 1], nn[lj])] += 1;
  }
}

__global__ void k_bc_fill(int N, const int4* __restrict__ tets, const int* __restrict__ ptr,
                          const int* __restrict__ ent, const int* __restrict__ row_ptr,
                          const int* __restrict__ cols, const int* __restrict__ bc_ptr, int* bc_cur,
                          int* bc_ent) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  for (int q = ptr[i]; q < ptr[i + 1]; ++q) {
    int t = ent[q] >> 2, li = ent[q] & 3;
    int4 n4 = tets[t];
    int nn[4] = {n4.x, n4.y, n4.z, n4.w};
    for (int lj = 0; lj < 4; ++lj) {
      int b = find_col(cols, row_ptr[i], row_ptr[i + 1], nn[lj]);
      bc_ent[bc_ptr[b] + bc_cur[b]++] = t * 16 + li * 4 + lj;
    }
  }
}

#define OT_TRY(x)                       \
  do {                                  \
    cudaError_t e_ = (x);               \
    if (e_ != cudaSuccess) return e_;   \
  } while (0)

}  // namespace

cudaError_t build_incidence(Context& c) {
  int* cnt = nullptr;
  OT_TRY(cudaMallocAsync(&cnt, sizeof(int) * (c.N + 1), c.stream));
  OT_TRY(cudaMemsetAsync(cnt, 0, sizeof(int) * (c.N + 1), c.stream));
  OT_TRY(cudaMallocAsync(&c.inc_ptr, sizeof(int) * (c.N + 1), c.stream));
  OT_TRY(cudaMallocAsync(&c.inc_ent, sizeof(int) * (4L * c.T + 1), c.stream));
  k_count_incidence<<<blocks_for(c.T), kThreads, 0, c.stream>>>(c.T, c.tets, cnt);
  OT_TRY(scan_exclusive(c, c.N, cnt, c.inc_ptr));
  OT_TRY(cudaMemsetAsync(cnt, 0, sizeof(int) * (c.N + 1), c.stream));
  k_fill_incidence<<<blocks_for(c.T), kThreads, 0, c.stream>>>(c.T, c.tets, c.inc_ptr, cnt, c.inc_ent);
  k_sort_incidence<<<(c.N + kSortWarps - 1) / kSortWarps, 32 * kSortWarps, 0, c.stream>>>(c.N, c.inc_ptr,
                                                                                         c.inc_ent);
  OT_TRY(cudaGetLastError());
  OT_TRY(cudaFreeAsync(cnt, c.stream));
  return cudaSuccess;
}

cudaError_t build_pattern(Context& c) {
  int *scratch = nullptr, *cnt = nullptr;
  OT_TRY(cudaMallocAsync(&scratch, sizeof(int) * (16L * c.T + 1), c.stream));
  OT_TRY(cudaMallocAsync(&cnt, sizeof(int) * (c.N + 1), c.stream));
  OT_TRY(cudaMallocAsync(&c.row_ptr, sizeof(int) * (c.N + 1), c.stream));
  k_row_unique<<<(c.N + kSortWarps - 1) / kSortWarps, 32 * kSortWarps, 0, c.stream>>>(c.N, c.tets, c.inc_ptr,
                                                                                     c.inc_ent, scratch, cnt);
  OT_TRY(scan_exclusive(c, c.N, cnt, c.row_ptr));
  int nnz = 0;
  OT_TRY(cudaMemcpyAsync(&nnz, c.row_ptr + c.N, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  OT_TRY(cudaStreamSynchronize(c.stream));
  c.nnz = nnz;
  OT_TRY(cudaMallocAsync(&c.cols, sizeof(int) * (c.nnz + 1), c.stream));
  k_row_fill<<<blocks_for(c.N), kThreads, 0, c.stream>>>(c.N, c.inc_ptr, scratch, c.row_ptr, c.cols);
  // block contribution lists
  int *bc_cnt = nullptr;
  OT_TRY(cudaMallocAsync(&bc_cnt, sizeof(int) * (c.nnz + 1), c.stream));
  OT_TRY(cudaMemsetAsync(bc_cnt, 0, sizeof(int) * (c.nnz + 1), c.stream));
  OT_TRY(cudaMallocAsync(&c.bc_ptr, sizeof(int) * (c.nnz + 1), c.stream));
  OT_TRY(cudaMallocAsync(&c.bc_ent, sizeof(int) * (16L * c.T + 1), c.stream));
  k_bc_count<<<blocks_for(c.N), kThreads, 0, c.stream>>>(c.N, c.tets, c.inc_ptr, c.inc_ent, c.row_ptr,
                                                         c.cols, bc_cnt);
  OT_TRY(scan_exclusive(c, c.nnz, bc_cnt, c.bc_ptr));
  OT_TRY(cudaMemsetAsync(bc_cnt, 0, sizeof(int) * (c.nnz + 1), c.stream));
  k_bc_fill<<<blocks_for(c.N), kThreads, 0, c.stream>>>(c.N, c.tets, c.inc_ptr, c.inc_ent, c.row_ptr,
                                                        c.cols, c.bc_ptr, bc_cnt, c.bc_ent);
  OT_TRY(cudaGetLastError());
  OT_TRY(cudaFreeAsync(bc_cnt, c.stream));
  OT_TRY(cudaFreeAsync(cnt, c.stream));
  OT_TRY(cudaFreeAsync(scratch, c.stream));
  return cudaSuccess;
}

// Exclusive prefix sum of n counts into out[0..n], out[n] = total (device,
// on the context's stream).
cudaError_t prefix_sum_counts(Context& c, long n, const int* in, int* out) { return scan_exclusive(c, n, in, out); }

}  // namespace otfem
