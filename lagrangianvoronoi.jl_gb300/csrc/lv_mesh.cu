// Re-binning and Voronoi clipping on the GPU: `remesh!`
// (src/voronoigrid.jl:89-108) and everything it calls.
//
// This translation unit is compiled with --fmad=false: every FP64 expression
// is evaluated as written, in the reference's order, so the polygons it
// produces are bit-identical to a sequential evaluation of
// src/polygon.jl:51-97 on the same candidate order.
//
// Pipeline (one stream, no host round trip):
//   k_bin_count    seed (+ periodic images) -> cell key, per-cell counts
//   scan           counts -> cell starts
//   k_bin_scatter  seed -> slot in its cells
//   k_bin_order    per cell: restore insertion (index) order, cache float2 positions
//   k_clip         one thread per polygon: candidate search along the cell path,
//                  half-plane clipping in shared memory, edge ordering, area,
//                  centroid and the interior-face quantities every operator uses.
#include <math.h>

#include "lv_internal.cuh"

namespace {

constexpr int SCAN_TPB = 256;
constexpr int SCAN_ITEMS = 4;  // per thread
constexpr int SCAN_TILE = SCAN_TPB * SCAN_ITEMS;

__device__ __forceinline__ int warp_incl_scan(int v) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) >= o) v += t;
  }
  return v;
}

// Block-wide exclusive scan of SCAN_TILE ints; writes the tile total.
__device__ void block_scan_tile(const int* in, int* out, int len, int base, int* tile_total) {
  __shared__ int warp_tot[SCAN_TPB / 32];
  int vals[SCAN_ITEMS];
  int sum = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    int idx = base + threadIdx.x * SCAN_ITEMS + k;
    vals[k] = (idx < len) ? in[idx] : 0;
    sum += vals[k];
  }
  int incl = warp_incl_scan(sum);
  if ((threadIdx.x & 31) == 31) warp_tot[threadIdx.x >> 5] = incl;
  __syncthreads();
  if (threadIdx.x < 32) {
    int t = (threadIdx.x < SCAN_TPB / 32) ? warp_tot[threadIdx.x] : 0;
    int ti = warp_incl_scan(t);
    if (threadIdx.x < SCAN_TPB / 32) warp_tot[threadIdx.x] = ti - t;
    if (threadIdx.x == SCAN_TPB / 32 - 1 && tile_total) *tile_total = ti;
  }
  __syncthreads();
  int run = warp_tot[threadIdx.x >> 5] + incl - sum;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    int idx = base + threadIdx.x * SCAN_ITEMS + k;
    if (idx < len) out[idx] = run;
    run += vals[k];
  }
}

__global__ void k_scan_tiles(const int* in, int* out, int len, int* tile_sums) {
  __shared__ int tot;
  block_scan_tile(in, out, len, blockIdx.x * SCAN_TILE, &tot);
  __syncthreads();
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

// Single block: exclusive scan of the tile sums (any count), total at [ntiles].
__global__ void k_scan_sums(int* sums, int ntiles) {
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < ntiles; base += SCAN_TILE) {
    __shared__ int tot;
    block_scan_tile(sums, sums, ntiles, base, &tot);
    __syncthreads();
    for (int k = threadIdx.x; k < SCAN_TILE && base + k < ntiles; k += blockDim.x) sums[base + k] += carry;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[ntiles] = carry;
}

__global__ void k_scan_add(int* out, int len, const int* sums, int ntiles) {
  int t = blockIdx.x;
  int add = sums[t];
  for (int k = threadIdx.x; k < SCAN_TILE; k += blockDim.x) {
    int idx = t * SCAN_TILE + k;
    if (idx < len) out[idx] += add;
  }
  if (t == 0 && threadIdx.x == 0) out[len] = sums[ntiles];
}

// ---------------------------------------------------------------- binning

// neighborlist.jl:47-52: key = floor((x - origin)/h) + 1, 1-based; returns
// the 0-based cell index or -1 when outside, -2 when not finite.
__device__ __forceinline__ int cell_of(const GridDev& g, double px, double py) {
  double dx = px - g.ox, dy = py - g.oy;
  double f1 = floor(dx / g.h), f2 = floor(dy / g.h);
  if (!(fabs(f1) < 1e15) || !(fabs(f2) < 1e15)) return -2;
  long long i1 = (long long)f1 + 1, i2 = (long long)f2 + 1;
  if (i1 < 1 || i1 > g.n1 || i2 < 1 || i2 > g.n2) return -1;
  return (int)((i1 - 1) + (long long)g.n1 * (i2 - 1));
}

// The 1, 3 or 9 copies inserted by insert_periodic! (voronoigrid.jl:130-147),
// in the reference's order.
__device__ __forceinline__ int image_count(const GridDev& g) {
  return 1 + (g.xper ? 2 : 0) + (g.yper ? 2 : 0) + ((g.xper && g.yper) ? 4 : 0);
}
__device__ __forceinline__ void image_pos(const GridDev& g, int k, double px, double py, double& qx, double& qy) {
  // order: x; x+X, x-X (xper); x+Y, x-Y (yper); x+X+Y, x+X-Y, x-X+Y, x-X-Y (both)
  int sx = 0, sy = 0;
  if (k > 0) {
    int kk = k - 1;
    if (g.xper) {
      if (kk < 2) { sx = kk == 0 ? 1 : -1; goto done; }
      kk -= 2;
    }
    if (g.yper) {
      if (kk < 2) { sy = kk == 0 ? 1 : -1; goto done; }
      kk -= 2;
    }
    sx = (kk < 2) ? 1 : -1;
    sy = (kk % 2 == 0) ? 1 : -1;
  }
done:
  qx = px;
  qy = py;
  if (sx > 0) qx = qx + g.xperiod;
  if (sx < 0) qx = qx - g.xperiod;
  if (sy > 0) qy = qy + g.yperiod;
  if (sy < 0) qy = qy - g.yperiod;
}

__global__ void k_bin_count(GridDev g, const double2* __restrict__ x, int n, int* ccount, int* status) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double2 p = x[i];
  int nim = image_count(g);
  for (int k = 0; k < nim; ++k) {
    double qx, qy;
    image_pos(g, k, p.x, p.y, qx, qy);
    int c = cell_of(g, qx, qy);
    if (c == -2) {
      atomicOr(status, LV_FLAG_NONFINITE);
      return;
    }
    if (c >= 0) atomicAdd(&ccount[c], 1);
  }
}

__global__ void k_bin_scatter(GridDev g, const double2* __restrict__ x, int n, const int* __restrict__ cstart,
                              int* cursor, int* citem, int item_cap, int* status) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double2 p = x[i];
  int nim = image_count(g);
  for (int k = 0; k < nim; ++k) {
    double qx, qy;
    image_pos(g, k, p.x, p.y, qx, qy);
    int c = cell_of(g, qx, qy);
    if (c < 0) continue;
    int slot = cstart[c] + atomicAdd(&cursor[c], 1);
    if (slot < item_cap)
      citem[slot] = i;
    else
      atomicOr(status, LV_FLAG_CELL_OVERFLOW);
  }
}

// Insertion order of the reference with one thread is the particle index
// order; atomics scatter arbitrarily, so each cell is sorted back.
__global__ void k_bin_order(int ncells, const int* __restrict__ cstart, int* citem, float2* cpos,
                            const double2* __restrict__ x, int item_cap) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  int a = cstart[c], b = min(cstart[c + 1], item_cap);
  for (int s = a + 1; s < b; ++s) {
    int v = citem[s];
    int t = s - 1;
    while (t >= a && citem[t] > v) {
      citem[t + 1] = citem[t];
      --t;
    }
    citem[t + 1] = v;
  }
  for (int s = a; s < b; ++s) {
    double2 p = x[citem[s]];
    cpos[s] = make_float2((float)p.x, (float)p.y);
  }
}

// ---------------------------------------------------------------- clipping

constexpr int CLIP_TPB = 64;
constexpr int ME = LV_MAX_EDGES;

struct Poly {
  double* v1x;
  double* v1y;
  double* v2x;
  double* v2y;
  int* lab;
  float* r32x;  // float copy of v1 - x, for the conservative prefilter
  float* r32y;
  int t;
  __device__ __forceinline__ int at(int k) const { return k * CLIP_TPB + t; }
};

__device__ __forceinline__ int signum_eps(double f) {  // polygon.jl:9-16
  return (f < -LV_SIGNUM_EPS) ? -1 : ((f > LV_SIGNUM_EPS) ? 1 : 0);
}

__device__ __forceinline__ double jmax(double a, double b) { return (b > a) ? b : a; }

// polygon.jl:101-107
__device__ double influence_rr(const Poly& P, int ne, double px, double py) {
  double rr = 0.0;
  for (int k = 0; k < ne; ++k) {
    double dx = P.v1x[P.at(k)] - px, dy = P.v1y[P.at(k)] - py;
    rr = jmax(rr, 4.0 * (dx * dx + dy * dy));
  }
  return rr;
}

__device__ __forceinline__ void refresh_r32(const Poly& P, int k, double px, double py) {
  P.r32x[P.at(k)] = (float)(P.v1x[P.at(k)] - px);
  P.r32y[P.at(k)] = (float)(P.v1y[P.at(k)] - py);
}

// polygon.jl:51-97, with FastVector's swap-delete (fastvector.jl:44-50).
// Returns 1 when a new edge was added, 0 otherwise, -1 on overflow.
__device__ int clip_halfplane(const Poly& P, int& ne, double px, double py, double yx, double yy, int label,
                               int& nev) {
  const double dfx = yx - px, dfy = yy - py;
  const double mx = 0.5 * (yx + px), my = 0.5 * (yy + py);
  const double c = dfx * mx + dfy * my;
  const double qnan = __longlong_as_double(0x7ff8000000000000LL);
  double Xx = qnan, Xy = qnan, Yx = qnan, Yy = qnan;
  int i = 0;
  while (i < ne) {
    const int a = P.at(i);
    const double a1x = P.v1x[a], a1y = P.v1y[a], a2x = P.v2x[a], a2y = P.v2y[a];
    const double f1 = dfx * a1x + dfy * a1y - c;
    const double f2 = dfx * a2x + dfy * a2y - c;
    const int s1 = signum_eps(f1), s2 = signum_eps(f2);
    const int s12 = s1 + s2;
    if (0 <= s12 && s12 <= 1 && (s1 | s2) != 0) {
      ++nev;
      Yx = Xx;
      Yy = Xy;
      const double inv = 1.0 / (f1 - f2);
      const double tx = f1 * a2x - f2 * a1x, ty = f1 * a2y - f2 * a1y;
      Xx = inv * tx;
      Xy = inv * ty;
      if (s1 == 0) { Xx = a1x; Xy = a1y; }
      if (s2 == 0) { Xx = a2x; Xy = a2y; }
      if (s1 == 1) {
        P.v1x[a] = Xx;
        P.v1y[a] = Xy;
        refresh_r32(P, i, px, py);
      } else {
        P.v2x[a] = Xx;
        P.v2y[a] = Xy;
      }
    }
    if (1 <= s12) {
      if (ne - 1 > i) {
        const int l = P.at(ne - 1);
        P.v1x[a] = P.v1x[l];
        P.v1y[a] = P.v1y[l];
        P.v2x[a] = P.v2x[l];
        P.v2y[a] = P.v2y[l];
        P.lab[a] = P.lab[l];
        P.r32x[a] = P.r32x[l];
        P.r32y[a] = P.r32y[l];
      }
      --ne;
    } else {
      ++i;
    }
  }
  const bool ynull = isnan(Yx) && isnan(Yy);
  if (!ynull && !(Xx == Yx && Xy == Yy)) {
    if (ne >= ME) return -1;
    const double ax = Yx - Xx, ay = Yy - Xy, bx = px - Xx, by = py - Xy;
    const int a = P.at(ne);
    if (ax * by - ay * bx > 0.0) {
      P.v1x[a] = Yx; P.v1y[a] = Yy; P.v2x[a] = Xx; P.v2y[a] = Xy;
    } else {
      P.v1x[a] = Xx; P.v1y[a] = Xy; P.v2x[a] = Yx; P.v2y[a] = Yy;
    }
    P.lab[a] = label;
    refresh_r32(P, ne, px, py);
    ++ne;
    return 1;
  }
  return 0;
}

// Conservative FP32 test: returns true only when the FP64 clip of this
// candidate provably changes nothing, i.e. every vertex v of the polygon has
// dot(y - x, v) - dot(y - x, (x + y)/2) < -SIGNUM_EPS in FP64.  d32 is the
// float offset y - x (error <= g.delta32 per component), the vertices are
// float offsets r = v - x (relative error 2^-24).  The bound covers the float
// rounding of d and r, the float arithmetic, and the FP64 rounding of the
// reference expression (which uses absolute coordinates up to g.bigm).
__device__ __forceinline__ bool prefilter_no_cut(const Poly& P, int ne, float dx, float dy, float rmax,
                                                 const GridDev& g) {
  const float d2 = dx * dx + dy * dy;
  const float D = sqrtf(d2) + 2.0f * g.delta32;
  const float R = rmax * 1.0001f;
  const float margin = 2.0f * g.delta32 * (R + 2.0f * D) + 4e-6f * (D * R + D * D) + 4e-15f * D * g.bigm + 1e-14f;
  const float half = 0.5f * d2;
  for (int k = 0; k < ne; ++k) {
    const float f = dx * P.r32x[P.at(k)] + dy * P.r32y[P.at(k)] - half;
    if (!(f < -margin)) return false;
  }
  return true;
}

// voronoigrid.jl:116-125
__device__ __forceinline__ void get_arrow(const GridDev& g, double ax, double ay, double bx, double by, double& vx,
                                          double& vy) {
  vx = ax - bx;
  vy = ay - by;
  if (g.xper && fabs(vx) > 0.5 * g.xperiod) vx -= (vx > 0 ? 1.0 : -1.0) * g.xperiod;
  if (g.yper && fabs(vy) > 0.5 * g.yperiod) vy -= (vy > 0 ? 1.0 : -1.0) * g.yperiod;
}

__device__ __forceinline__ bool veq_bits(double a, double b) { return a == b; }

__global__ void __launch_bounds__(CLIP_TPB) k_clip(GridDev g, const PathNodeDev* __restrict__ path,
                                                   const double2* __restrict__ x, int n, CellsDev cl, MeshDev m,
                                                   int* status, int use_prefilter) {
  extern __shared__ double smem[];
  const int t = threadIdx.x;
  const int i = blockIdx.x * CLIP_TPB + t;
  Poly P;
  P.v1x = smem;
  P.v1y = P.v1x + ME * CLIP_TPB;
  P.v2x = P.v1y + ME * CLIP_TPB;
  P.v2y = P.v2x + ME * CLIP_TPB;
  P.lab = reinterpret_cast<int*>(P.v2y + ME * CLIP_TPB);
  P.r32x = reinterpret_cast<float*>(P.lab + ME * CLIP_TPB);
  P.r32y = P.r32x + ME * CLIP_TPB;
  P.t = t;
  if (i >= n) return;

  const double2 xi = x[i];
  const double px = xi.x, py = xi.y;
  // reset! (polygon.jl:37-47): the cropping rectangle, edges B->A, A->D, D->C, C->B
  {
    const double Ax = g.cminx, Ay = g.cminy, Cx = g.cmaxx, Cy = g.cmaxy;
    const double Bx = Cx, By = Ay, Dx = Ax, Dy = Cy;
    const double e1[4][4] = {{Bx, By, Ax, Ay}, {Ax, Ay, Dx, Dy}, {Dx, Dy, Cx, Cy}, {Cx, Cy, Bx, By}};
    const int labs[4] = {LV_BDARY_DOWN, LV_BDARY_LEFT, LV_BDARY_UP, LV_BDARY_RIGHT};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int a = P.at(k);
      P.v1x[a] = e1[k][0];
      P.v1y[a] = e1[k][1];
      P.v2x[a] = e1[k][2];
      P.v2y[a] = e1[k][3];
      P.lab[a] = labs[k];
      refresh_r32(P, k, px, py);
    }
  }
  int ne = 4;
  int flag = 0;
  double prr = influence_rr(P, ne, px, py);
  const double dxo = px - g.ox, dyo = py - g.oy;
  const double f1 = floor(dxo / g.h), f2 = floor(dyo / g.h);
  if (!(fabs(f1) < 1e15) || !(fabs(f2) < 1e15)) {
    flag = LV_FLAG_NONFINITE;
  } else {
    const long long k1 = (long long)f1 + 1, k2 = (long long)f2 + 1;
    // The float prefilter assumes the polygon's edges form a closed chain, so
    // that the v1 vertices are all the vertices.  A clip with other than
    // exactly two crossing events (degenerate input) can open the chain; the
    // prefilter is then switched off for this polygon.
    bool chain_ok = true;
    const float x32 = (float)px, y32 = (float)py;
    const float xp32 = (float)g.xperiod, yp32 = (float)g.yperiod;
    // voronoigrid.jl:53-81
    for (int pn = 0; pn < g.npath; ++pn) {
      const double rr = path[pn].rr;
      if (rr > prr) break;
      if (rr > g.rr_max) {
        flag = LV_FLAG_MESH_DESTROYED;
        break;
      }
      const long long c1 = k1 + path[pn].di1, c2 = k2 + path[pn].di2;
      if (c1 < 1 || c1 > g.n1 || c2 < 1 || c2 > g.n2) continue;
      const int cell = (int)((c1 - 1) + (long long)g.n1 * (c2 - 1));
      const int sa = cl.cstart[cell], sb = cl.cstart[cell + 1];
      for (int s = sa; s < sb; ++s) {
        const int j = cl.citem[s];
        if (j == i) continue;  // y == x exactly: get_arrow(x, x) = 0
        if (use_prefilter && chain_ok) {
          const float2 q32 = cl.cpos[s];
          float ddx = q32.x - x32, ddy = q32.y - y32;
          bool far_image = false;
          if (g.xper) {
            if (fabsf(ddx) > 0.45f * xp32) far_image = true;
          }
          if (g.yper) {
            if (fabsf(ddy) > 0.45f * yp32) far_image = true;
          }
          if (!far_image) {
            // distance test norm_squared(x - y) > prr, decided in float when unambiguous
            const float d2 = ddx * ddx + ddy * ddy;
            const float dd = sqrtf(d2);
            const float prr32 = (float)prr;
            const float lo = d2 * (1.0f - 1e-6f) - 4.0f * g.delta32 * dd - 4.0f * g.delta32 * g.delta32;
            if (lo > prr32 * (1.0f + 1e-6f)) continue;
            const float rmax = 0.5f * sqrtf(prr32) * (1.0f + 1e-6f);
            if (prefilter_no_cut(P, ne, ddx, ddy, rmax, g)) continue;
          }
        }
        const double2 xq = x[j];
        double vx, vy;
        get_arrow(g, xq.x, xq.y, px, py, vx, vy);
        const double yx = px + vx, yy = py + vy;
        if (veq_bits(px, yx) && veq_bits(py, yy)) continue;
        const double ex = px - yx, ey = py - yy;
        if (ex * ex + ey * ey > prr) continue;
        int nev = 0;
        const int r = clip_halfplane(P, ne, px, py, yx, yy, j, nev);
        if (nev != 0 && !(r == 1 && nev == 2)) chain_ok = false;
        if (r < 0) {
          flag = LV_FLAG_EDGE_OVERFLOW;
          break;
        }
        if (r) prr = influence_rr(P, ne, px, py);
      }
      if (flag) break;
    }
  }
  if (flag) atomicOr(status, flag);

  // sort_edges! (IO.jl:35-48)
  for (int a = 0; a < ne; ++a) {
    const double lx = P.v2x[P.at(a)], ly = P.v2y[P.at(a)];
    for (int b = a + 1; b < ne; ++b) {
      if (lx == P.v1x[P.at(b)] && ly == P.v1y[P.at(b)]) {
        const int u = P.at(a + 1), w = P.at(b);
        double t0;
        int tl;
        t0 = P.v1x[u]; P.v1x[u] = P.v1x[w]; P.v1x[w] = t0;
        t0 = P.v1y[u]; P.v1y[u] = P.v1y[w]; P.v1y[w] = t0;
        t0 = P.v2x[u]; P.v2x[u] = P.v2x[w]; P.v2x[w] = t0;
        t0 = P.v2y[u]; P.v2y[u] = P.v2y[w]; P.v2y[w] = t0;
        tl = P.lab[u]; P.lab[u] = P.lab[w]; P.lab[w] = tl;
        break;
      }
    }
  }

  // area (polygon.jl:114-121), centroid (polygon.jl:210-219), faces.
  double A = 0.0, Ac = 0.0, cx = 0.0, cy = 0.0;
  int nf = 0;
  const int cap = m.cap;
  for (int k = 0; k < ne; ++k) {
    const int a = P.at(k);
    const double v1x = P.v1x[a], v1y = P.v1y[a], v2x = P.v2x[a], v2y = P.v2y[a];
    const int lab = P.lab[a];
    const double ax = v1x - px, ay = v1y - py, bx = v2x - px, by = v2y - py;
    const double dA = 0.5 * fabs(ax * by - ay * bx);
    A += dA;
    Ac += dA;
    const double sx = (px + v1x) + v2x, sy = (py + v1y) + v2y;
    cx = cx + (dA * sx) / 3.0;
    cy = cy + (dA * sy) / 3.0;
    m.ev1[(size_t)k * cap + i] = make_double2(v1x, v1y);
    m.ev2[(size_t)k * cap + i] = make_double2(v2x, v2y);
    m.elab[(size_t)k * cap + i] = lab;
    if (lab >= 0) {
      const double2 xq = x[lab];
      double vx, vy;
      get_arrow(g, xq.x, xq.y, px, py, vx, vy);
      const double yx = px + vx, yy = py + vy;
      const double lx = v1x - v2x, ly = v1y - v2y;
      const double l2 = lx * lx + ly * ly;
      const double rx = px - yx, ry = py - yy;
      const double r2 = rx * rx + ry * ry;
      const size_t f = (size_t)nf * cap + i;
      m.fnbr[f] = lab;
      m.flrr[f] = sqrt(l2 / r2);
      m.flen[f] = sqrt(lx * lx + ly * ly);
      m.fm[f] = make_double2(0.5 * (v1x + v2x), 0.5 * (v1y + v2y));
      m.fy[f] = make_double2(yx, yy);
      ++nf;
    }
  }
  m.nedges[i] = ne;
  m.nfaces[i] = nf;
  m.area[i] = A;
  m.centroid[i] = make_double2(cx / Ac, cy / Ac);
}

}  // namespace

int lv_scan_int(lv_ctx* c, const int* in, int* out, int len) {
  int ntiles = (len + SCAN_TILE - 1) / SCAN_TILE;
  if (ntiles == 0) {
    cudaMemsetAsync(out, 0, sizeof(int), c->stream);
    return LV_OK;
  }
  int* sums = reinterpret_cast<int*>(c->sv.tmp);  // scratch, >= ntiles + 1 ints
  k_scan_tiles<<<ntiles, SCAN_TPB, 0, c->stream>>>(in, out, len, sums);
  LV_LAUNCH_CHECK(c, "k_scan_tiles");
  k_scan_sums<<<1, SCAN_TPB, 0, c->stream>>>(sums, ntiles);
  LV_LAUNCH_CHECK(c, "k_scan_sums");
  k_scan_add<<<ntiles, SCAN_TPB, 0, c->stream>>>(out, len, sums, ntiles);
  LV_LAUNCH_CHECK(c, "k_scan_add");
  return LV_OK;
}

int lv_mesh_remesh(lv_ctx* c) {
  const int n = c->n;
  if (n <= 0) return lv_fail(c, LV_ERR_NOT_MESHED, "remesh: no particles");
  cudaStream_t s = c->stream;
  const int nc = c->c.ncells;
  {
  KernelTimer kt(c, LV_KF_BIN);
  cudaMemsetAsync(c->c.ccount, 0, sizeof(int) * nc, s);
  k_bin_count<<<lv_blocks(n, 256), 256, 0, s>>>(c->g, c->s.x, n, c->c.ccount, c->status);
  LV_LAUNCH_CHECK(c, "k_bin_count");
  int rc = lv_scan_int(c, c->c.ccount, c->c.cstart, nc);
  if (rc) return rc;
  cudaMemsetAsync(c->c.ccount, 0, sizeof(int) * nc, s);
  k_bin_scatter<<<lv_blocks(n, 256), 256, 0, s>>>(c->g, c->s.x, n, c->c.cstart, c->c.ccount, c->c.citem,
                                                    c->c.item_cap, c->status);
  LV_LAUNCH_CHECK(c, "k_bin_scatter");
  k_bin_order<<<lv_blocks(nc, 256), 256, 0, s>>>(nc, c->c.cstart, c->c.citem, c->c.cpos, c->s.x, c->c.item_cap);
  LV_LAUNCH_CHECK(c, "k_bin_order");
  }
  const size_t smem = (size_t)ME * CLIP_TPB * (4 * sizeof(double) + sizeof(int) + 2 * sizeof(float));
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_clip, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr_set = true;
  }
  {
    KernelTimer kt(c, LV_KF_CLIP);
    k_clip<<<lv_blocks(n, CLIP_TPB), CLIP_TPB, smem, s>>>(c->g, c->path, c->s.x, n, c->c, c->m, c->status, 1);
    LV_LAUNCH_CHECK(c, "k_clip");
  }
  c->meshed = true;
  c->op_ready = false;
  return LV_OK;
}
