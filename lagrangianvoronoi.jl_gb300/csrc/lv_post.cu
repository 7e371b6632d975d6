// Post-processing on the device mesh (movingls.jl, voronoigrid.jl:154-178):
// nearest_polygon, movingls (linear / quadratic / cubic Taylor expansion by
// Gaussian-weighted moving least squares) and point_value.  One thread per
// query; every query walks the reference's cell path over the cell list as
// the reference's loops do.  Compiled with --fmad=false like the geometry.
#include <algorithm>
#include <cmath>
#include <vector>

#include "lv_internal.cuh"

namespace {

__device__ __forceinline__ bool findkey(const GridDev& g, double px, double py, long long& k1, long long& k2) {
  const double f1 = floor((px - g.ox) / g.h), f2 = floor((py - g.oy) / g.h);
  if (!(fabs(f1) < 1e15) || !(fabs(f2) < 1e15)) return false;
  k1 = (long long)f1 + 1;
  k2 = (long long)f2 + 1;
  return true;
}

__device__ __forceinline__ void arrow(const GridDev& g, double ax, double ay, double bx, double by, double& vx,
                                      double& vy) {  // voronoigrid.jl:116-125
  vx = ax - bx;
  vy = ay - by;
  if (g.xper && fabs(vx) > 0.5 * g.xperiod) vx -= (vx > 0 ? 1.0 : -1.0) * g.xperiod;
  if (g.yper && fabs(vy) > 0.5 * g.yperiod) vy -= (vy > 0 ? 1.0 : -1.0) * g.yperiod;
}

// voronoigrid.jl:154-178; -1 when the path prefix meets no polygon
__device__ int nearest(const GridDev& g, const PathNodeDev* __restrict__ path, int npath, const CellsDev& cl,
                       const double2* __restrict__ x, double qx, double qy) {
  long long k1, k2;
  if (!findkey(g, qx, qy, k1, k2)) return -1;
  double rr_best = INFINITY;
  int best = -1;
  for (int pn = 0; pn < npath; ++pn) {
    if (path[pn].rr > rr_best) break;
    const long long c1 = k1 + path[pn].di1, c2 = k2 + path[pn].di2;
    if (c1 < 1 || c1 > g.n1 || c2 < 1 || c2 > g.n2) continue;
    const int cell = (int)((c1 - 1) + (long long)g.n1 * (c2 - 1));
    for (int s = cl.cstart[cell], se = min(cl.cstart[cell + 1], cl.item_cap); s < se; ++s) {
      const int i = cl.citem[s];
      const double2 p = x[i];
      const double dx = p.x - qx, dy = p.y - qy;
      const double prr = dx * dx + dy * dy;
      if (prr < rr_best) {
        rr_best = prr;
        best = i;
      }
    }
  }
  return best;
}

template <int NC>
__device__ void power_vec(double dx, double dy, double* pv) {  // movingls.jl:26-36
  pv[0] = dx;
  pv[1] = dy;
  if (NC >= 5) {
    pv[2] = dx * dx;
    pv[3] = dx * dy;
    pv[4] = dy * dy;
  }
  if (NC >= 9) {
    pv[5] = (dx * dx) * dx;
    pv[6] = (dx * dx) * dy;
    pv[7] = (dx * dy) * dy;
    pv[8] = (dy * dy) * dy;
  }
}

// R \ a: the explicit 2x2 formula, Gaussian elimination with partial pivoting otherwise
template <int NC>
__device__ void small_solve(double* R, double* a) {
  if constexpr (NC == 2) {
    const double d = R[0] * R[3] - R[2] * R[1];
    const double b0 = a[0], b1 = a[1];
    a[0] = (R[3] * b0 - R[2] * b1) / d;
    a[1] = (R[0] * b1 - R[1] * b0) / d;
    return;
  } else {
  for (int k = 0; k < NC; ++k) {
    int piv = k;
    for (int r = k + 1; r < NC; ++r)
      if (fabs(R[r + NC * k]) > fabs(R[piv + NC * k])) piv = r;
    if (piv != k) {
      for (int c = 0; c < NC; ++c) {
        const double t = R[k + NC * c];
        R[k + NC * c] = R[piv + NC * c];
        R[piv + NC * c] = t;
      }
      const double t = a[k];
      a[k] = a[piv];
      a[piv] = t;
    }
    for (int r = k + 1; r < NC; ++r) {
      const double f = R[r + NC * k] / R[k + NC * k];
      for (int c = k; c < NC; ++c) R[r + NC * c] -= f * R[k + NC * c];
      a[r] -= f * a[k];
    }
  }
  for (int k = NC - 1; k >= 0; --k) {
    double t = a[k];
    for (int c = k + 1; c < NC; ++c) t -= R[k + NC * c] * a[c];
    a[k] = t / R[k + NC * k];
  }
  }
}

// movingls (movingls.jl:52-86), gaussian_kernel (:22-24), polygon i
template <int NC>
__device__ void movingls(const GridDev& g, const PathNodeDev* __restrict__ path, int npath, const CellsDev& cl,
                         const double2* __restrict__ x, const double* __restrict__ f, int i, double h,
                         double* out) {
  double a[NC], R[NC * NC], pv[NC];
  for (int k = 0; k < NC; ++k) a[k] = 0.0;
  for (int k = 0; k < NC * NC; ++k) R[k] = 0.0;
  const double2 p = x[i];
  const double fp = f[i];
  long long k1, k2;
  if (findkey(g, p.x, p.y, k1, k2)) {
    for (int pn = 0; pn < npath; ++pn) {
      if (path[pn].rr > h) break;
      const long long c1 = k1 + path[pn].di1, c2 = k2 + path[pn].di2;
      if (c1 < 1 || c1 > g.n1 || c2 < 1 || c2 > g.n2) continue;
      const int cell = (int)((c1 - 1) + (long long)g.n1 * (c2 - 1));
      for (int s = cl.cstart[cell], se = min(cl.cstart[cell + 1], cl.item_cap); s < se; ++s) {
        const int j = cl.citem[s];
        const double2 q = x[j];
        double vx, vy;
        arrow(g, q.x, q.y, p.x, p.y, vx, vy);
        const double yx = p.x + vx, yy = p.y + vy;
        if (p.x == yx && p.y == yy) continue;
        const double rx = p.x - yx, ry = p.y - yy;
        const double r = sqrt(rx * rx + ry * ry);
        if (r < h) {
          const double qq = r / h;
          const double ker = exp(-0.5 * (qq * qq)) / sqrt((2.0 * M_PI) * (h * h));
          power_vec<NC>(yx - p.x, yy - p.y, pv);
          const double sc = ker * (f[j] - fp);
          for (int k = 0; k < NC; ++k) a[k] += sc * pv[k];
          for (int l = 0; l < NC; ++l)
            for (int k = 0; k < NC; ++k) R[k + NC * l] += (ker * pv[k]) * pv[l];
        }
      }
    }
  }
  small_solve<NC>(R, a);
  for (int k = 0; k < NC; ++k) out[k] = a[k];
}

__global__ void k_nearest(GridDev g, const PathNodeDev* __restrict__ path, int npath, CellsDev cl,
                          const double2* __restrict__ x, int m, const double2* __restrict__ q, int* out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < m) out[t] = nearest(g, path, npath, cl, x, q[t].x, q[t].y);
}

template <int NC>
__global__ void k_movingls(GridDev g, const PathNodeDev* __restrict__ path, int npath, CellsDev cl,
                           const double2* __restrict__ x, const double* __restrict__ f, int m,
                           const int* __restrict__ polys, double h, double* out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < m) movingls<NC>(g, path, npath, cl, x, f, polys ? polys[t] : t, h, out + (size_t)NC * t);
}

// point_value (movingls.jl:140-146): nearest polygon, linear expansion, h = grid.h
__global__ void k_point_value(GridDev g, const PathNodeDev* __restrict__ pnear, int nnear,
                              const PathNodeDev* __restrict__ pls, int nls, CellsDev cl,
                              const double2* __restrict__ x, const double* __restrict__ f, int m,
                              const double2* __restrict__ q, double* out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  const int i = nearest(g, pnear, nnear, cl, x, q[t].x, q[t].y);
  if (i < 0) {
    out[t] = NAN;
    return;
  }
  double L[2];
  movingls<2>(g, pls, nls, cl, x, f, i, g.h, L);
  const double2 p = x[i];
  out[t] = f[i] + (L[0] * (q[t].x - p.x) + L[1] * (q[t].y - p.y));
}

// The reference's cell path (neighborlist.jl:29-41) ordered like lv_create's
// prefix, up to the first node with rr > bound, within the grid's offset range.
std::vector<PathNodeDev> path_upto(const GridDev& g, double bound) {
  struct Node {
    long long i1, i2, keysq;
    double rr;
  };
  std::vector<Node> all;
  for (long long i2 = 1 - (long long)g.n1; i2 <= g.n1 - 1; ++i2)
    for (long long i1 = 1 - (long long)g.n2; i1 <= g.n2 - 1; ++i1) {
      const long long a = std::max<long long>(0, llabs(i1) - 1), b = std::max<long long>(0, llabs(i2) - 1);
      volatile double hh = g.h * g.h;
      const double rr = hh * (double)(a * a + b * b);
      if (rr > bound && rr > 4.0 * bound + 16.0 * hh) continue;  // far beyond the cut: never visited
      all.push_back({i1, i2, i1 * i1 + i2 * i2, rr});
    }
  std::stable_sort(all.begin(), all.end(), [](const Node& p, const Node& q) { return p.keysq < q.keysq; });
  std::stable_sort(all.begin(), all.end(), [](const Node& p, const Node& q) { return p.rr < q.rr; });
  std::vector<PathNodeDev> out;
  for (const auto& nd : all) {
    out.push_back(PathNodeDev{(int)nd.i1, (int)nd.i2, nd.rr, (float)nd.rr, nd.rr > bound ? 1 : 0});
    if (nd.rr > bound) break;
  }
  return out;
}

struct DevBuf {
  void* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

}  // namespace

extern "C" {

int lv_nearest_polygon(lv_ctx* c, int32_t m, const double* points, int32_t* out) {
  if (!c || m < 0 || (m > 0 && (!points || !out))) return LV_ERR_BAD_ARGUMENT;
  if (!c->meshed) return lv_fail(c, LV_ERR_NOT_MESHED, "the grid has not been meshed");
  if (m == 0) return LV_OK;
  DevBuf q, o;
  if (cudaMalloc(&q.p, 16 * (size_t)m) != cudaSuccess || cudaMalloc(&o.p, 4 * (size_t)m) != cudaSuccess)
    return lv_fail(c, LV_ERR_CUDA, "lv_nearest_polygon: allocation failed");
  cudaMemcpyAsync(q.p, points, 16 * (size_t)m, cudaMemcpyHostToDevice, c->stream);
  k_nearest<<<lv_blocks(m, 128), 128, 0, c->stream>>>(c->g, c->path, c->g.npath, c->c, c->s.x, m,
                                                      static_cast<const double2*>(q.p), static_cast<int*>(o.p));
  c->launches++;
  cudaMemcpyAsync(out, o.p, 4 * (size_t)m, cudaMemcpyDeviceToHost, c->stream);
  return lv_cuda_check(c, cudaStreamSynchronize(c->stream), "lv_nearest_polygon");
}

int lv_movingls(lv_ctx* c, int32_t order, int32_t m, const int32_t* polys, const double* values, double h,
                double* coeffs) {
  if (!c || order < 1 || order > 3 || m < 0 || !values || !coeffs || !(h > 0)) return LV_ERR_BAD_ARGUMENT;
  if (!c->meshed) return lv_fail(c, LV_ERR_NOT_MESHED, "the grid has not been meshed");
  const int n = c->n;
  if (!polys && m != n) return lv_fail(c, LV_ERR_BAD_ARGUMENT, "lv_movingls: m must equal n when polys is NULL");
  if (polys)
    for (int k = 0; k < m; ++k)
      if (polys[k] < 0 || polys[k] >= n) return lv_fail(c, LV_ERR_BAD_ARGUMENT, "lv_movingls: polygon out of range");
  if (m == 0) return LV_OK;
  const int nc = order == 1 ? 2 : (order == 2 ? 5 : 9);
  const std::vector<PathNodeDev> path = path_upto(c->g, h);
  DevBuf dp, df, dpl, dout;
  bool ok = cudaMalloc(&dp.p, sizeof(PathNodeDev) * path.size()) == cudaSuccess;
  ok = ok && cudaMalloc(&df.p, 8 * (size_t)n) == cudaSuccess;
  ok = ok && (!polys || cudaMalloc(&dpl.p, 4 * (size_t)m) == cudaSuccess);
  ok = ok && cudaMalloc(&dout.p, 8 * (size_t)nc * m) == cudaSuccess;
  if (!ok) return lv_fail(c, LV_ERR_CUDA, "lv_movingls: allocation failed");
  cudaStream_t s = c->stream;
  cudaMemcpyAsync(dp.p, path.data(), sizeof(PathNodeDev) * path.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(df.p, values, 8 * (size_t)n, cudaMemcpyHostToDevice, s);
  if (polys) cudaMemcpyAsync(dpl.p, polys, 4 * (size_t)m, cudaMemcpyHostToDevice, s);
  const PathNodeDev* P = static_cast<const PathNodeDev*>(dp.p);
  const int np = (int)path.size();
  const double* F = static_cast<const double*>(df.p);
  const int* PL = static_cast<const int*>(dpl.p);
  double* O = static_cast<double*>(dout.p);
  const int nb = lv_blocks(m, 128);
  if (nc == 2) k_movingls<2><<<nb, 128, 0, s>>>(c->g, P, np, c->c, c->s.x, F, m, PL, h, O);
  else if (nc == 5) k_movingls<5><<<nb, 128, 0, s>>>(c->g, P, np, c->c, c->s.x, F, m, PL, h, O);
  else k_movingls<9><<<nb, 128, 0, s>>>(c->g, P, np, c->c, c->s.x, F, m, PL, h, O);
  c->launches++;
  cudaMemcpyAsync(coeffs, O, 8 * (size_t)nc * m, cudaMemcpyDeviceToHost, s);
  return lv_cuda_check(c, cudaStreamSynchronize(s), "lv_movingls");
}

int lv_point_value(lv_ctx* c, int32_t m, const double* points, const double* values, double* out) {
  if (!c || m < 0 || (m > 0 && (!points || !values || !out))) return LV_ERR_BAD_ARGUMENT;
  if (!c->meshed) return lv_fail(c, LV_ERR_NOT_MESHED, "the grid has not been meshed");
  if (m == 0) return LV_OK;
  const int n = c->n;
  const std::vector<PathNodeDev> path = path_upto(c->g, c->g.h);
  DevBuf dp, df, dq, dout;
  bool ok = cudaMalloc(&dp.p, sizeof(PathNodeDev) * path.size()) == cudaSuccess;
  ok = ok && cudaMalloc(&df.p, 8 * (size_t)n) == cudaSuccess;
  ok = ok && cudaMalloc(&dq.p, 16 * (size_t)m) == cudaSuccess;
  ok = ok && cudaMalloc(&dout.p, 8 * (size_t)m) == cudaSuccess;
  if (!ok) return lv_fail(c, LV_ERR_CUDA, "lv_point_value: allocation failed");
  cudaStream_t s = c->stream;
  cudaMemcpyAsync(dp.p, path.data(), sizeof(PathNodeDev) * path.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(df.p, values, 8 * (size_t)n, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dq.p, points, 16 * (size_t)m, cudaMemcpyHostToDevice, s);
  k_point_value<<<lv_blocks(m, 128), 128, 0, s>>>(c->g, c->path, c->g.npath, static_cast<const PathNodeDev*>(dp.p),
                                                  (int)path.size(), c->c, c->s.x, static_cast<const double*>(df.p),
                                                  m, static_cast<const double2*>(dq.p),
                                                  static_cast<double*>(dout.p));
  c->launches++;
  cudaMemcpyAsync(out, dout.p, 8 * (size_t)m, cudaMemcpyDeviceToHost, s);
  return lv_cuda_check(c, cudaStreamSynchronize(s), "lv_point_value");
}

}  // extern "C"
