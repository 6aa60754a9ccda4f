// otfem_coupling.cu -- mesh coupling of a surface point set to the volume
// mesh (t4mesh::mesh_coupling, t4mesh_mesh_coupling.h): binding each point to
// a tet that contains it and moving the points with the deformed tets.
//
// Binding (bind_surface, :129-236): a point is embedded in a tet when all
// four barycentric weights lie in (-1e-4, 1 + 1e-4) (collision_policy::
// report, :84-111), with the weights of geometry::barycentric_algebraic for
// tetrahedra (geometry_barycentric.h:343-385): w = P^-1 (p - x_m) with the
// columns of P the edges x_i - x_m, x_j - x_m, x_k - x_m, and w_m = 1 - sum.
// The reference finds candidate tets with a spatial hash and keeps the first
// tet reported; here a uniform grid over the mesh's bounding box holds every
// tet in the cells its bounding box overlaps, and a point takes the lowest
// tet index that embeds it (a fixed choice; on a shared face both tets give
// the same position up to rounding, the interpolation being continuous).
// A point no tet embeds stays unbound, as in the reference, and keeps its
// position.
//
// Update (update_surface, :238-275): p = w0 x_i + w1 x_j + w2 x_k + w3 x_m
// with w0 = 1 - w1 - w2 - w3 and the stored (w1, w2, w3), the reference's
// `barycentric` entries, in the reference's order of operations.
#include <algorithm>
#include <cmath>
#include <vector>

#include "otfem_internal.h"

using otfem::Context;

struct otfem_surface_s {
  Context* c = nullptr;  // the volume mesh (its handle must outlive the surface)
  int64_t count = 0;
  int32_t* tet = nullptr;    // bound tet per point, -1: none
  double* bary = nullptr;    // 3 per point: (w1, w2, w3)
  double* rest = nullptr;    // 3 per point: the points as given
};

namespace otfem {
namespace {

constexpr double kBaryDelta = 10e-5;  // t4mesh_mesh_coupling.h:91

struct Grid {
  double lo[3], inv_h;
  int n[3];
};

__device__ __forceinline__ int cell_coord(const Grid& g, double v, int d) {
  int k = int(floor((v - g.lo[d]) * g.inv_h));
  return k < 0 ? 0 : (k >= g.n[d] ? g.n[d] - 1 : k);
}

// The cells a tet's bounding box overlaps (widened by a margin for the
// tolerance of the embedding test).
__device__ __forceinline__ void tet_cells(const Grid& g, const int4& n, const double* __restrict__ x, double margin,
                                          int (&c0)[3], int (&c1)[3]) {
  const int id[4] = {n.x, n.y, n.z, n.w};
  for (int d = 0; d < 3; ++d) {
    double mn = x[3L * id[0] + d], mx = mn;
    for (int k = 1; k < 4; ++k) {
      const double v = x[3L * id[k] + d];
      mn = fmin(mn, v);
      mx = fmax(mx, v);
    }
    c0[d] = cell_coord(g, mn - margin, d);
    c1[d] = cell_coord(g, mx + margin, d);
  }
}

__global__ void k_grid_count(int T, const int4* __restrict__ tets, const double* __restrict__ x, Grid g, double margin,
                             int* count) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  int c0[3], c1[3];
  tet_cells(g, tets[t], x, margin, c0, c1);
  for (int a = c0[0]; a <= c1[0]; ++a)
    for (int b = c0[1]; b <= c1[1]; ++b)
      for (int d = c0[2]; d <= c1[2]; ++d) atomicAdd(&count[(long(a) * g.n[1] + b) * g.n[2] + d], 1);
}

__global__ void k_grid_fill(int T, const int4* __restrict__ tets, const double* __restrict__ x, Grid g, double margin,
                            const int* __restrict__ start, int* cursor, int* cell_tets) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  int c0[3], c1[3];
  tet_cells(g, tets[t], x, margin, c0, c1);
  for (int a = c0[0]; a <= c1[0]; ++a)
    for (int b = c0[1]; b <= c1[1]; ++b)
      for (int d = c0[2]; d <= c1[2]; ++d) {
        const long cell = (long(a) * g.n[1] + b) * g.n[2] + d;
        cell_tets[start[cell] + atomicAdd(&cursor[cell], 1)] = t;
      }
}

// geometry_barycentric.h:343-385 for the tet (x_i, x_j, x_k, x_m): the
// weights of x_i, x_j, x_k; x_m's is 1 minus their sum.
__device__ __forceinline__ void tet_barycentric(const double* xi, const double* xj, const double* xk, const double* xm,
                                                const double* p, double (&w)[4]) {
  double P[3][3], r[3];
  for (int d = 0; d < 3; ++d) {
    P[d][0] = xi[d] - xm[d];
    P[d][1] = xj[d] - xm[d];
    P[d][2] = xk[d] - xm[d];
    r[d] = p[d] - xm[d];
  }
  // P^-1 = adj(P) / det(P)
  const double c00 = P[1][1] * P[2][2] - P[1][2] * P[2][1];
  const double c01 = P[1][2] * P[2][0] - P[1][0] * P[2][2];
  const double c02 = P[1][0] * P[2][1] - P[1][1] * P[2][0];
  const double det = P[0][0] * c00 + P[0][1] * c01 + P[0][2] * c02;
  const double inv = 1.0 / det;
  const double i00 = c00 * inv, i01 = (P[0][2] * P[2][1] - P[0][1] * P[2][2]) * inv,
               i02 = (P[0][1] * P[1][2] - P[0][2] * P[1][1]) * inv;
  const double i10 = c01 * inv, i11 = (P[0][0] * P[2][2] - P[0][2] * P[2][0]) * inv,
               i12 = (P[0][2] * P[1][0] - P[0][0] * P[1][2]) * inv;
  const double i20 = c02 * inv, i21 = (P[0][1] * P[2][0] - P[0][0] * P[2][1]) * inv,
               i22 = (P[0][0] * P[1][1] - P[0][1] * P[1][0]) * inv;
  w[0] = i00 * r[0] + i01 * r[1] + i02 * r[2];
  w[1] = i10 * r[0] + i11 * r[1] + i12 * r[2];
  w[2] = i20 * r[0] + i21 * r[1] + i22 * r[2];
  w[3] = 1.0 - w[0] - w[1] - w[2];
}

__global__ void k_bind_points(long P, const double* __restrict__ pts, int T, const int4* __restrict__ tets,
                              const double* __restrict__ x, Grid g, const int* __restrict__ start,
                              const int* __restrict__ cell_tets, int32_t* tet_out, double* bary_out) {
  const long i = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= P) return;
  const double p[3] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
  int best = -1;
  double wb[4] = {0.0, 0.0, 0.0, 0.0};
  bool inside = true;
  for (int d = 0; d < 3; ++d) {
    const double k = (p[d] - g.lo[d]) * g.inv_h;
    if (!(k >= -1.0 && k <= double(g.n[d]) + 1.0)) inside = false;  // also NaN
  }
  if (inside) {
    const long cell = (long(cell_coord(g, p[0], 0)) * g.n[1] + cell_coord(g, p[1], 1)) * g.n[2] + cell_coord(g, p[2], 2);
    const double lower = -kBaryDelta, upper = 1.0 + kBaryDelta;
    for (int q = start[cell]; q < start[cell + 1]; ++q) {
      const int t = cell_tets[q];
      if (best >= 0 && t >= best) continue;
      const int4 n = tets[t];
      double w[4];
      tet_barycentric(x + 3L * n.x, x + 3L * n.y, x + 3L * n.z, x + 3L * n.w, p, w);
      if (w[0] > lower && w[0] < upper && w[1] > lower && w[1] < upper && w[2] > lower && w[2] < upper &&
          w[3] > lower && w[3] < upper) {
        best = t;
        for (int k = 0; k < 4; ++k) wb[k] = w[k];
      }
    }
  }
  tet_out[i] = best;
  // bind_surface keeps (m_w1, m_w2, m_w3): the weights of x_j, x_k, x_m
  bary_out[3 * i] = wb[1];
  bary_out[3 * i + 1] = wb[2];
  bary_out[3 * i + 2] = wb[3];
}

__global__ void k_update_points(long P, const int32_t* __restrict__ tet, const double* __restrict__ bary,
                                const double* __restrict__ rest, const int4* __restrict__ tets,
                                const double* __restrict__ x, double* out) {
  const long i = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= P) return;
  const int t = tet[i];
  if (t < 0) {
    for (int d = 0; d < 3; ++d) out[3 * i + d] = rest[3 * i + d];
    return;
  }
  const int4 n = tets[t];
  const double w1 = bary[3 * i], w2 = bary[3 * i + 1], w3 = bary[3 * i + 2];
  const double w0 = 1.0 - w1 - w2 - w3;
  for (int d = 0; d < 3; ++d) {
    // p0*w0 + p1*w1 + p2*w2 + p3*w3, left to right (t4mesh_mesh_coupling.h:272)
    const double s = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(x[3L * n.x + d], w0), __dmul_rn(x[3L * n.y + d], w1)),
                                         __dmul_rn(x[3L * n.z + d], w2)),
                               __dmul_rn(x[3L * n.w + d], w3));
    out[3 * i + d] = s;
  }
}

}  // namespace
}  // namespace otfem

namespace {
void free_surface(otfem_surface_s* s) {
  if (!s) return;
  cudaFree(s->tet);
  cudaFree(s->bary);
  cudaFree(s->rest);
  delete s;
}
}  // namespace

extern "C" {

int otfem_surface_bind(otfem_handle h, const double* points, int64_t count, otfem_surface* out, int64_t* bound) {
  using namespace otfem;
  if (!h || !out || (!points && count > 0) || count < 0)
    return record_error(OTFEM_ERR_INVALID_ARGUMENT, "null argument or negative count");
  *out = nullptr;
  Context& c = *context_of(h);
  if (!c.initialized) return record_error(OTFEM_ERR_NOT_INITIALIZED, "otfem_init has not been called");
  for (int64_t i = 0; i < 3 * count; ++i)
    if (!std::isfinite(points[i])) return record_error(OTFEM_ERR_INVALID_ARGUMENT, "non-finite point");
  auto* s = new otfem_surface_s;
  s->c = &c;
  s->count = count;
  cudaError_t e = cudaSuccess;
  auto fail_cuda = [&](const char* what) {
    free_surface(s);
    return record_error(OTFEM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  };
  const size_t P = size_t(std::max<int64_t>(count, 1));
  if ((e = cudaMalloc(&s->tet, sizeof(int32_t) * P)) != cudaSuccess) return fail_cuda("cudaMalloc");
  if ((e = cudaMalloc(&s->bary, sizeof(double) * 3 * P)) != cudaSuccess) return fail_cuda("cudaMalloc");
  if ((e = cudaMalloc(&s->rest, sizeof(double) * 3 * P)) != cudaSuccess) return fail_cuda("cudaMalloc");
  if (count > 0 &&
      (e = cudaMemcpyAsync(s->rest, points, sizeof(double) * 3 * count, cudaMemcpyHostToDevice, c.stream)) !=
          cudaSuccess)
    return fail_cuda("upload points");
  // the grid: the current node coordinates' bounding box, cells of about one
  // tet's size, at most 4 T cells
  std::vector<double> xh(3 * size_t(c.N));
  if (c.N && (e = cudaMemcpyAsync(xh.data(), c.x, sizeof(double) * xh.size(), cudaMemcpyDeviceToHost, c.stream)) !=
                 cudaSuccess)
    return fail_cuda("download coordinates");
  if ((e = cudaStreamSynchronize(c.stream)) != cudaSuccess) return fail_cuda("synchronize");
  Grid g{};
  double hi[3];
  for (int d = 0; d < 3; ++d) {
    g.lo[d] = c.N ? xh[d] : 0.0;
    hi[d] = g.lo[d];
  }
  for (int i = 0; i < c.N; ++i)
    for (int d = 0; d < 3; ++d) {
      g.lo[d] = std::min(g.lo[d], xh[3 * size_t(i) + d]);
      hi[d] = std::max(hi[d], xh[3 * size_t(i) + d]);
    }
  double ext[3], vol = 1.0;
  for (int d = 0; d < 3; ++d) {
    ext[d] = std::max(hi[d] - g.lo[d], 1e-12);
    vol *= ext[d];
  }
  const double T = std::max(c.T, 1);
  double cell = std::cbrt(vol / T);
  for (int d = 0; d < 3; ++d) cell = std::max(cell, ext[d] / 1024.0);
  long cells = 1;
  for (;;) {
    cells = 1;
    for (int d = 0; d < 3; ++d) {
      g.n[d] = std::max(1, int(std::ceil(ext[d] / cell)));
      cells *= g.n[d];
    }
    if (cells <= 4 * long(T) + 1) break;
    cell *= 1.25;
  }
  g.inv_h = 1.0 / cell;
  const double margin = 1e-3 * cell;
  int *count_d = nullptr, *start = nullptr, *cell_tets = nullptr;
  auto cleanup = [&]() {
    cudaFree(count_d);
    cudaFree(start);
    cudaFree(cell_tets);
  };
  if ((e = cudaMalloc(&count_d, sizeof(int) * (cells + 1))) != cudaSuccess) return cleanup(), fail_cuda("cudaMalloc");
  if ((e = cudaMalloc(&start, sizeof(int) * (cells + 1))) != cudaSuccess) return cleanup(), fail_cuda("cudaMalloc");
  cudaMemsetAsync(count_d, 0, sizeof(int) * (cells + 1), c.stream);
  const int tb = (c.T + 255) / 256 > 0 ? (c.T + 255) / 256 : 1;
  if (c.T > 0) k_grid_count<<<tb, 256, 0, c.stream>>>(c.T, c.tets, c.x, g, margin, count_d);
  if ((e = cudaGetLastError()) != cudaSuccess) return cleanup(), fail_cuda("grid count");
  if ((e = prefix_sum_counts(c, cells, count_d, start)) != cudaSuccess) return cleanup(), fail_cuda("grid scan");
  int entries = 0;
  if ((e = cudaMemcpyAsync(&entries, start + cells, sizeof(int), cudaMemcpyDeviceToHost, c.stream)) != cudaSuccess ||
      (e = cudaStreamSynchronize(c.stream)) != cudaSuccess)
    return cleanup(), fail_cuda("grid size");
  if ((e = cudaMalloc(&cell_tets, sizeof(int) * std::max(entries, 1))) != cudaSuccess)
    return cleanup(), fail_cuda("cudaMalloc");
  cudaMemsetAsync(count_d, 0, sizeof(int) * (cells + 1), c.stream);
  if (c.T > 0) k_grid_fill<<<tb, 256, 0, c.stream>>>(c.T, c.tets, c.x, g, margin, start, count_d, cell_tets);
  if (count > 0)
    k_bind_points<<<unsigned((count + 255) / 256), 256, 0, c.stream>>>(count, s->rest, c.T, c.tets, c.x, g, start,
                                                                      cell_tets, s->tet, s->bary);
  if ((e = cudaGetLastError()) != cudaSuccess) return cleanup(), fail_cuda("bind");
  std::vector<int32_t> th(P);
  if (count > 0 &&
      (e = cudaMemcpyAsync(th.data(), s->tet, sizeof(int32_t) * count, cudaMemcpyDeviceToHost, c.stream)) !=
          cudaSuccess)
    return cleanup(), fail_cuda("download binding");
  if ((e = cudaStreamSynchronize(c.stream)) != cudaSuccess) return cleanup(), fail_cuda("synchronize");
  cleanup();
  if (bound) *bound = std::count_if(th.begin(), th.begin() + count, [](int32_t t) { return t >= 0; });
  *out = s;
  return OTFEM_OK;
}

int otfem_surface_update_device(otfem_surface s, double* device_out, int64_t count) {
  using namespace otfem;
  if (!s || (!device_out && count > 0)) return record_error(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  if (count != s->count) return record_error(OTFEM_ERR_INVALID_ARGUMENT, "count does not match the bound points");
  if (count == 0) return OTFEM_OK;
  Context& c = *s->c;
  k_update_points<<<unsigned((count + 255) / 256), 256, 0, c.stream>>>(count, s->tet, s->bary, s->rest, c.tets, c.x,
                                                                      device_out);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return record_error(OTFEM_ERR_CUDA, std::string("update: ") + cudaGetErrorString(e));
  c.launches += 1;
  return OTFEM_OK;
}

int otfem_surface_update(otfem_surface s, double* host_out, int64_t count) {
  using namespace otfem;
  if (!s || (!host_out && count > 0)) return record_error(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  if (count != s->count) return record_error(OTFEM_ERR_INVALID_ARGUMENT, "count does not match the bound points");
  if (count == 0) return OTFEM_OK;
  Context& c = *s->c;
  double* d = nullptr;
  cudaError_t e = cudaMallocAsync(&d, sizeof(double) * 3 * size_t(count), c.stream);
  if (e != cudaSuccess) return record_error(OTFEM_ERR_CUDA, std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
  int rc = otfem_surface_update_device(s, d, count);
  if (rc == OTFEM_OK) {
    e = cudaMemcpyAsync(host_out, d, sizeof(double) * 3 * size_t(count), cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaFreeAsync(d, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) rc = record_error(OTFEM_ERR_CUDA, std::string("update: ") + cudaGetErrorString(e));
  } else {
    cudaFreeAsync(d, c.stream);
  }
  return rc;
}

int otfem_surface_binding(otfem_surface s, int32_t* tet, double* barycentric, int64_t count) {
  using namespace otfem;
  if (!s) return record_error(OTFEM_ERR_INVALID_ARGUMENT, "null surface");
  if (count != s->count) return record_error(OTFEM_ERR_INVALID_ARGUMENT, "count does not match the bound points");
  if (count == 0) return OTFEM_OK;
  Context& c = *s->c;
  cudaError_t e = cudaSuccess;
  if (tet) e = cudaMemcpyAsync(tet, s->tet, sizeof(int32_t) * count, cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess && barycentric)
    e = cudaMemcpyAsync(barycentric, s->bary, sizeof(double) * 3 * count, cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) return record_error(OTFEM_ERR_CUDA, std::string("binding: ") + cudaGetErrorString(e));
  return OTFEM_OK;
}

int otfem_surface_destroy(otfem_surface s) {
  if (!s) return OTFEM_OK;
  cudaStreamSynchronize(s->c->stream);
  free_surface(s);
  return OTFEM_OK;
}

}  // extern "C"
