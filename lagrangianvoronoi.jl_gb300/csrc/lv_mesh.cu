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
//                  centroid and the interior-face quantities every operator uses
//   k_clip_redo    the polygons that outgrew the first pass's edge slots,
//                  resumed from their captures with LV_MAX_EDGES slots
#include <math.h>
#include <stdlib.h>

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
// quick: the position is a periodic image of a finite one, and positions
// surely outside the grid skip the divisions: dx < 0 gives floor(dx/h) <= -1,
// dx >= dx_hi gives floor(dx/h) >= n1 (most images of a periodic domain).
__device__ __forceinline__ int cell_of(const GridDev& g, double px, double py, bool quick) {
  double dx = px - g.ox, dy = py - g.oy;
  if (quick && (dx < 0.0 || dy < 0.0 || dx >= g.dx_hi || dy >= g.dy_hi)) return -1;
  double f1 = floor(div_rcp(dx, g.h, g.rh)), f2 = floor(div_rcp(dy, g.h, g.rh));
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
// the period shifts (sx, sy) of copy k, in the order
// x; x+X, x-X (xper); x+Y, x-Y (yper); x+X+Y, x+X-Y, x-X+Y, x-X-Y (both)
__device__ __forceinline__ void image_shift(const GridDev& g, int k, int& sx, int& sy) {
  sx = 0;
  sy = 0;
  if (k == 0) return;
  int kk = k - 1;
  if (g.xper) {
    if (kk < 2) {
      sx = kk == 0 ? 1 : -1;
      return;
    }
    kk -= 2;
  }
  if (g.yper) {
    if (kk < 2) {
      sy = kk == 0 ? 1 : -1;
      return;
    }
    kk -= 2;
  }
  sx = (kk < 2) ? 1 : -1;
  sy = (kk % 2 == 0) ? 1 : -1;
}
__device__ __forceinline__ void image_pos(const GridDev& g, int k, double px, double py, double& qx, double& qy) {
  int sx, sy;
  image_shift(g, k, sx, sy);
  qx = px;
  qy = py;
  if (sx > 0) qx = qx + g.xperiod;
  if (sx < 0) qx = qx - g.xperiod;
  if (sy > 0) qy = qy + g.yperiod;
  if (sy < 0) qy = qy - g.yperiod;
}

// Counts every copy per cell and keeps, per copy k of particle i, its cell
// and its rank among the cell's copies in key[k * cap + i] (cell -1: outside
// the grid), so that the scatter needs neither the cell computation nor
// atomics.
__global__ void k_bin_count(GridDev g, const double2* __restrict__ x, int n, int cap, int* ccount, int2* key,
                            int* status, int* redo_n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) *redo_n = 0;  // the clipping pass's capture count, for this remesh
  if (i >= n) return;
  double2 p = x[i];
  int nim = image_count(g);
  // x- (y-) shifted images of a position well inside the domain lie outside
  // the grid (decided in float, skipping their FP64 position and cell tests)
  const float fx = (float)p.x, fy = (float)p.y;
  const bool farx = fx > g.ixlo && fx < g.ixhi, fary = fy > g.iylo && fy < g.iyhi;
  for (int k = 0; k < nim; ++k) {
    if (k > 0 && (farx || fary)) {
      int sx, sy;
      image_shift(g, k, sx, sy);
      if ((sx != 0 && farx) || (sy != 0 && fary)) {
        key[(size_t)k * cap + i] = make_int2(-1, 0);
        continue;
      }
    }
    double qx, qy;
    image_pos(g, k, p.x, p.y, qx, qy);
    int c = cell_of(g, qx, qy, k > 0);
    if (c == -2) {
      atomicOr(status, LV_FLAG_NONFINITE);
      for (; k < nim; ++k) key[(size_t)k * cap + i] = make_int2(-1, 0);
      return;
    }
    key[(size_t)k * cap + i] = make_int2(c, c >= 0 ? atomicAdd(&ccount[c], 1) : 0);
  }
}

__global__ void k_bin_scatter(GridDev g, int n, int cap, const int2* __restrict__ key, const int* __restrict__ cstart,
                              int* citem, int item_cap, int* status) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int nim = image_count(g);
  for (int k = 0; k < nim; ++k) {
    const int2 cr = key[(size_t)k * cap + i];
    if (cr.x < 0) continue;
    int slot = cstart[cr.x] + cr.y;
    if (slot < item_cap)
      citem[slot] = i;
    else
      atomicOr(status, LV_FLAG_CELL_OVERFLOW);
  }
}

// Insertion order of the reference with one thread is the particle index
// order; atomics scatter arbitrarily, so each cell is sorted back.  Each item
// then gets the float offset of its particle from the cell's lower corner
// (the clipping's float tests; an offset below h carries an error of 2^-24 h
// instead of 2^-24 of the coordinate), or NaN when the item is a periodic
// image (its copy 0, the particle itself, lies in another cell), which the
// clipping decides in FP64.
// (also clears the cell counts for the next remesh: the scan has consumed them)
__global__ void k_bin_order(GridDev g, const int2* __restrict__ key, int ncells, const int* __restrict__ cstart,
                            int* citem, float2* cpos, const double2* __restrict__ x, int item_cap, int* ccount) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  ccount[c] = 0;
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
  const double ox = g.ox + (double)(c % g.n1) * g.h, oy = g.oy + (double)(c / g.n1) * g.h;
  const float qnan = __int_as_float(0x7fc00000);
  for (int s = a; s < b; ++s) {
    const int i = citem[s];
    if (key[i].x == c) {
      const double2 p = x[i];
      cpos[s] = make_float2((float)(p.x - ox), (float)(p.y - oy));
    } else {
      cpos[s] = make_float2(qnan, qnan);
    }
  }
}

// ---------------------------------------------------------------- clipping
//
// One thread per polygon (FP64 work is priced per warp instruction on this
// GPU, so full warps of independent polygons use the FP64 pipe best).  The
// polygon lives in shared memory in the reference's edge order.  Besides the
// FP64 edges each slot keeps float offsets of both vertices from the seed
// (from which a float upper bound of 4|v1 - x|^2 is formed), so that:
//  * a candidate's fate is decided in float whenever that is provably
//    exact: "cannot cut" (all vertices strictly inside the half-plane with a
//    margin covering every rounding) is skipped, and vertex signs away from
//    the bisector come from float; only vertices within the margin and the
//    two crossing edges (whose intersection must be exact) are evaluated in
//    FP64 with the reference's expressions;
//  * a candidate's offset from the seed is formed in float from offsets to
//    the cell corners (stored by the binning) and the path node's cell
//    offset, so its error scales with the cell size, not with the coordinates;
//  * the influence radius is an upper bound, which can only admit extra
//    candidates that cannot cut (no-ops), and is replaced by the exact FP64
//    value where the reference's "mesh destroyed" test needs it;
//  * work is done in rounds: every thread first advances through its
//    candidates with float/integer work until it meets one that may cut, then
//    the warp performs the FP64 clips of that round together.
// Any case the float path cannot certify (a clip with other than two
// crossing edges) runs the reference's clip verbatim in FP64.

constexpr int CLIP_TPB = 64;
constexpr int ME = LV_MAX_EDGES;
// edge slots of the first clipping pass: shared memory for 8 edges per
// polygon (52 bytes a slot) lets eight blocks share an SM (three with
// LV_MAX_EDGES); a polygon that needs more at any point is captured and
// finished by a second pass with LV_MAX_EDGES slots, spread over every SM.
// Measured on Taylor-Green meshes (256^2 / 1024^2, ms per remesh x2),
// before the warp-uniform clip: 8 slots 1.84 / 12.9, 10 slots 1.44 / 12.8,
// 12 slots 1.49 / 14.2, 14 slots 1.52 / 16.6, all 20 slots in one pass
// 1.93 / 20.9; with it: 10 slots 1.274 / 10.44, 9 slots 1.271 / 10.16; with
// the second pass spread over every SM: 9 slots 1.123 / 9.58, 8 slots (eight
// blocks per SM) 1.140 / 9.08; with the second pass resuming the captured
// polygons: 9 slots 1.054 / 9.92, 8 slots 1.122 / 10.29.  On the 4M double
// shear with the clip-count order and the register-cached scan: 9 slots
// 24.5, 8 slots (eight blocks per SM) 24.0 ms per step.
constexpr int ME_SMALL = 8;

struct Poly {
  double* v1x;
  double* v1y;
  double* v2x;
  double* v2y;
  int* lab;
  float* r1x;  // v1 - x (float)
  float* r1y;
  float* r2x;  // v2 - x (float)
  float* r2y;
  int t;
  int cap_e;   // edge slots
  __device__ __forceinline__ int at(int k) const { return k * CLIP_TPB + t; }
};

// a == b (IEEE) decided on the integer pipe: equal bit patterns of a value
// that is not NaN, or two zeros of either sign.
__device__ __forceinline__ bool same_value(double a, double b) {
  const unsigned long long x = (unsigned long long)__double_as_longlong(a);
  const unsigned long long y = (unsigned long long)__double_as_longlong(b);
  constexpr unsigned long long MAG = 0x7fffffffffffffffull;
  return (x == y && (x & MAG) <= 0x7ff0000000000000ull) || ((x | y) & MAG) == 0ull;
}

// RN(a / 3) with one multiplication and two fused multiply-adds (Markstein,
// IBM J. Res. Dev. 34(1), 1990): y = RN(1/3) = (1/3)(1 - 2^-54) lies within
// half an ulp of 1/3, so q = RN(a y) lies within one ulp of a/3, the residual
// r = a - 3q is exact in one fma, and RN(q + r y) is the correctly rounded
// quotient.  For |a| outside [2^-900, 2^1000) (zeros, values whose residual
// could be subnormal, infinities, NaN) the division itself.
__device__ __forceinline__ double div3(double a) {
  const unsigned ex = ((unsigned)__double2hiint(a) >> 20) & 0x7ffu;
  if (ex - 123u < 1900u) {
    const double y = 0x1.5555555555555p-2;
    const double q = a * y;
    const double r = fma(-3.0, q, a);
    return fma(r, y, q);
  }
  return a / 3.0;
}

__device__ __forceinline__ int signum_eps(double f) {  // polygon.jl:9-16
  return (f < -LV_SIGNUM_EPS) ? -1 : ((f > LV_SIGNUM_EPS) ? 1 : 0);
}

// float upper bound of 4 (dx^2 + dy^2) for a float pair already rounded
// from the FP64 offset (relative error <= 2^-24 each)
__device__ __forceinline__ float d2_up(float dx, float dy) { return 4.0f * (dx * dx + dy * dy) * (1.0f + 1e-6f); }

__device__ __forceinline__ void set_v1(const Poly& P, int k, double vx, double vy, double px, double py) {
  const int a = P.at(k);
  P.v1x[a] = vx;
  P.v1y[a] = vy;
  const float fx = (float)(vx - px), fy = (float)(vy - py);
  P.r1x[a] = fx;
  P.r1y[a] = fy;
}

__device__ __forceinline__ void set_v2(const Poly& P, int k, double vx, double vy, double px, double py) {
  const int a = P.at(k);
  P.v2x[a] = vx;
  P.v2y[a] = vy;
  P.r2x[a] = (float)(vx - px);
  P.r2y[a] = (float)(vy - py);
}

__device__ __forceinline__ void copy_slot(const Poly& P, int dst, int src) {
  const int a = P.at(dst), l = P.at(src);
  P.v1x[a] = P.v1x[l];
  P.v1y[a] = P.v1y[l];
  P.v2x[a] = P.v2x[l];
  P.v2y[a] = P.v2y[l];
  P.lab[a] = P.lab[l];
  P.r1x[a] = P.r1x[l];
  P.r1y[a] = P.r1y[l];
  P.r2x[a] = P.r2x[l];
  P.r2y[a] = P.r2y[l];
}

// polygon.jl:101-107, exact
__device__ double influence_rr_exact(const Poly& P, int ne, double px, double py) {
  double rr = 0.0;
  for (int k = 0; k < ne; ++k) {
    const double dx = P.v1x[P.at(k)] - px, dy = P.v1y[P.at(k)] - py;
    const double t = 4.0 * (dx * dx + dy * dy);
    rr = (t > rr) ? t : rr;
  }
  return rr;
}

// The new edge (X, Y) of a clip, oriented counter-clockwise about the seed
// and appended in the next slot (polygon.jl:88-95).
__device__ __forceinline__ void append_edge(const Poly& P, int& ne, double Xx, double Xy, double Yx, double Yy,
                                            double px, double py, int label) {
  const double ax = Yx - Xx, ay = Yy - Xy, bx = px - Xx, by = py - Xy;
  if (ax * by - ay * bx > 0.0) {
    set_v1(P, ne, Yx, Yy, px, py);
    set_v2(P, ne, Xx, Xy, px, py);
  } else {
    set_v1(P, ne, Xx, Xy, px, py);
    set_v2(P, ne, Yx, Yy, px, py);
  }
  P.lab[P.at(ne)] = label;
  ++ne;
}

// the points of a new edge that found no free slot
struct PendingEdge {
  double xx, xy, yx, yy;
};

// polygon.jl:51-97 verbatim in FP64, with FastVector's swap-delete
// (fastvector.jl:44-50).  Returns 1 when a new edge was added, 0 otherwise,
// -1 when the new edge finds no free slot (its points then go to pend, the
// polygon's other edges being final); nev counts crossing events.
__device__ int clip_exact(const Poly& P, int& ne, double px, double py, double yx, double yy, int label, int& nev,
                          PendingEdge& pend) {
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
      if (s1 == 1)
        set_v1(P, i, Xx, Xy, px, py);
      else
        set_v2(P, i, Xx, Xy, px, py);
    }
    if (1 <= s12) {
      if (ne - 1 > i) copy_slot(P, i, ne - 1);
      --ne;
    } else {
      ++i;
    }
  }
  const bool ynull = isnan(Yx) && isnan(Yy);
  if (!ynull && !(same_value(Xx, Yx) && same_value(Xy, Yy))) {
    if (ne >= P.cap_e) {
      pend = PendingEdge{Xx, Xy, Yx, Yy};
      return -1;
    }
    append_edge(P, ne, Xx, Xy, Yx, Yy, px, py, label);
    return 1;
  }
  return 0;
}

// Same result as clip_exact (bit for bit) for the common case of exactly two
// crossing edges.  Returns 2 when it cannot certify the case (the caller then
// runs clip_exact on the unchanged polygon), otherwise as clip_exact.
//
// Vertex signs: f32 = d.r - |d|^2/2 with d = float(y - x) and r the stored
// float offset; the FP64 value f of the reference differs from the exact
// value of f32's expression by at most 2^-24-relative rounding of d, r and
// the float arithmetic (<= 1e-6 (D R + D^2) with D = |d|, R >= |r|) plus the
// FP64 rounding of the reference expression in absolute coordinates
// (<= 4e-15 D M, M = max |coordinate|), so |f32| > that margin + 2 eps
// decides signum(f) exactly; otherwise f is evaluated in FP64.
//
// FP64 work is priced per warp instruction, so it is laid out for the warp:
// the pass over the edges only classifies (float, FP64 just for vertices
// within the margin); the vertex values of the two crossing edges, their
// intersection points and the float offsets of those points are then
// computed by every lane with the same instructions, and written to the slots
// through selects instead of branches.  The values are the same expressions
// as the reference's, so the result is unchanged.
__device__ __forceinline__ void put_vertex(const Poly& P, int k, bool first, double vx, double vy, float fx,
                                           float fy) {
  const int a = P.at(k);
  double* X = first ? P.v1x : P.v2x;
  double* Y = first ? P.v1y : P.v2y;
  float* RX = first ? P.r1x : P.r2x;
  float* RY = first ? P.r1y : P.r2y;
  X[a] = vx;
  Y[a] = vy;
  RX[a] = fx;
  RY[a] = fy;
}

__device__ int clip_fast(const Poly& P, int& ne, double px, double py, double yx, double yy, int label, float bigm,
                         PendingEdge& pend) {
  const double dfx = yx - px, dfy = yy - py;
  const double mx = 0.5 * (yx + px), my = 0.5 * (yy + py);
  const double c = dfx * mx + dfy * my;
  const float dx = (float)dfx, dy = (float)dfy;
  const float dd2 = dx * dx + dy * dy;
  const float D = sqrtf(dd2) * 1.0001f;
  float R = 0.0f;
  for (int k = 0; k < ne; ++k) R = fmaxf(R, d2_up(P.r1x[P.at(k)], P.r1y[P.at(k)]));
  R = 0.5f * sqrtf(R) * 1.0001f;
  const float margin = 1e-6f * (D * R + D * D) + 4e-15f * D * bigm + 1e-14f;
  const float half = 0.5f * dd2;
  // classification: per-edge code 0 keep, 1 event-keep, 2 event-delete, 3 delete
  unsigned long long code = 0ull;  // 2 bits per slot
  int nev = 0;
  int e0_slot = 0, e1_slot = 0, e0_s1 = 0, e0_s2 = 0, e1_s1 = 0, e1_s2 = 0;
  for (int k = 0; k < ne; ++k) {
    const int a = P.at(k);
    const float g1 = dx * P.r1x[a] + dy * P.r1y[a] - half;
    const float g2 = dx * P.r2x[a] + dy * P.r2y[a] - half;
    int s1, s2;
    if (g1 < -margin) s1 = -1;
    else if (g1 > margin) s1 = 1;
    else s1 = signum_eps(dfx * P.v1x[a] + dfy * P.v1y[a] - c);
    if (g2 < -margin) s2 = -1;
    else if (g2 > margin) s2 = 1;
    else s2 = signum_eps(dfx * P.v2x[a] + dfy * P.v2y[a] - c);
    const int s12 = s1 + s2;
    unsigned cd = 0;
    if (0 <= s12 && s12 <= 1 && (s1 | s2) != 0) {
      if (nev >= 2) return 2;
      if (nev == 0) {
        e0_slot = k; e0_s1 = s1; e0_s2 = s2;
      } else {
        e1_slot = k; e1_s1 = s1; e1_s2 = s2;
      }
      ++nev;
      cd = (s12 >= 1) ? 2u : 1u;
    } else if (s12 >= 1) {
      cd = 3u;
    }
    code |= (unsigned long long)cd << (2 * k);
  }
  if (nev == 0) {
    if (code != 0ull) return 2;  // deletions without crossings: degenerate
    return 0;
  }
  if (nev != 2) return 2;
  // the crossing edges' vertex values and intersection points (original
  // data).  Their vertices have s1 != s2 in sign or one zero, so f1 != f2.
  double X0x, X0y, X1x, X1y;
  {
    const int a = P.at(e0_slot);
    const double a1x = P.v1x[a], a1y = P.v1y[a], a2x = P.v2x[a], a2y = P.v2y[a];
    const double f1 = dfx * a1x + dfy * a1y - c;
    const double f2 = dfx * a2x + dfy * a2y - c;
    const double inv = 1.0 / (f1 - f2);
    X0x = inv * (f1 * a2x - f2 * a1x);
    X0y = inv * (f1 * a2y - f2 * a1y);
    if (e0_s1 == 0) { X0x = a1x; X0y = a1y; }
    if (e0_s2 == 0) { X0x = a2x; X0y = a2y; }
  }
  {
    const int a = P.at(e1_slot);
    const double a1x = P.v1x[a], a1y = P.v1y[a], a2x = P.v2x[a], a2y = P.v2y[a];
    const double f1 = dfx * a1x + dfy * a1y - c;
    const double f2 = dfx * a2x + dfy * a2y - c;
    const double inv = 1.0 / (f1 - f2);
    X1x = inv * (f1 * a2x - f2 * a1x);
    X1y = inv * (f1 * a2y - f2 * a1y);
    if (e1_s1 == 0) { X1x = a1x; X1y = a1y; }
    if (e1_s2 == 0) { X1x = a2x; X1y = a2y; }
  }
  const float q0x = (float)(X0x - px), q0y = (float)(X0y - py);
  const float q1x = (float)(X1x - px), q1y = (float)(X1y - py);
  // the reference's sequential pass over the slots with swap-delete; the
  // crossing identity (2 bits: 0 none, 1 first, 2 second in slot order)
  // travels with its slot.
  unsigned long long ident = (1ull << (2 * e0_slot)) | (2ull << (2 * e1_slot));
  int visited_first = 0, visited_last = 0;  // crossing id (1 or 2) visited first / last
  int fs0 = -1, fs1 = -1;                  // final slot of a kept crossing
  int i = 0;
  int nn = ne;
  while (i < nn) {
    const unsigned cd = (unsigned)((code >> (2 * i)) & 3ull);
    const unsigned id = (unsigned)((ident >> (2 * i)) & 3ull);
    if (id) {
      if (visited_first == 0) visited_first = (int)id;
      else visited_last = (int)id;
    }
    if (cd >= 2u) {
      if (nn - 1 > i) {
        copy_slot(P, i, nn - 1);
        const unsigned long long lastc = (code >> (2 * (nn - 1))) & 3ull;
        const unsigned long long lasti = (ident >> (2 * (nn - 1))) & 3ull;
        code = (code & ~(3ull << (2 * i))) | (lastc << (2 * i));
        ident = (ident & ~(3ull << (2 * i))) | (lasti << (2 * i));
      }
      --nn;
    } else {
      if (id == 1) fs0 = i;
      if (id == 2) fs1 = i;
      ++i;
    }
  }
  // a kept crossing edge: its outside vertex becomes the intersection point
  if (fs0 >= 0) put_vertex(P, fs0, e0_s1 == 1, X0x, X0y, q0x, q0y);
  if (fs1 >= 0) put_vertex(P, fs1, e1_s1 == 1, X1x, X1y, q1x, q1y);
  ne = nn;
  // new edge from X = the crossing visited last, Y = the one visited first
  const bool xl0 = visited_last == 1, yf0 = visited_first == 1;
  const double Xx = xl0 ? X0x : X1x, Xy = xl0 ? X0y : X1y;
  const double Yx = yf0 ? X0x : X1x, Yy = yf0 ? X0y : X1y;
  if (same_value(Xx, Yx) && same_value(Xy, Yy)) return 0;
  if (ne >= P.cap_e) {
    pend = PendingEdge{Xx, Xy, Yx, Yy};
    return -1;
  }
  const float rXx = xl0 ? q0x : q1x, rXy = xl0 ? q0y : q1y;
  const float rYx = yf0 ? q0x : q1x, rYy = yf0 ? q0y : q1y;
  // reorient counter-clockwise (Y -> X) when the reference's FP64
  // (Y - X) x (p - X) > 0.  That product equals (X - p) x (Y - p), which the
  // float offsets give to within 1e-6 of |rXx rYy| + |rXy rYx| (their 2^-24
  // roundings and the float arithmetic) plus the FP64 rounding of the
  // reference's expression (a few 1e-16 of the squared offsets); outside
  // that margin its sign decides, otherwise the reference's expression does.
  const float cf = rXx * rYy - rXy * rYx;
  const float mo = 1e-6f * (fabsf(rXx * rYy) + fabsf(rXy * rYx)) +
                   1e-14f * ((rXx * rXx + rXy * rXy) + (rYx * rYx + rYy * rYy)) + 1e-30f;
  bool inv = cf > 0.0f;
  if (!(fabsf(cf) > mo)) {
    const double ax = Yx - Xx, ay = Yy - Xy, bx = px - Xx, by = py - Xy;
    inv = ax * by - ay * bx > 0.0;
  }
  put_vertex(P, ne, true, inv ? Yx : Xx, inv ? Yy : Xy, inv ? rYx : rXx, inv ? rYy : rXy);
  put_vertex(P, ne, false, inv ? Xx : Yx, inv ? Xy : Yy, inv ? rXx : rYx, inv ? rXy : rYy);
  P.lab[P.at(ne)] = label;
  ++ne;
  return 1;
}

// voronoigrid.jl:116-125
__device__ __forceinline__ void get_arrow(const GridDev& g, double ax, double ay, double bx, double by, double& vx,
                                          double& vy) {
  vx = ax - bx;
  vy = ay - by;
  // fabs(v) > 0.5 * period, compared on the integer pipe (the wrap is rare)
  if (g.xper && abs_greater(vx, g.hxbits)) vx -= (vx > 0 ? 1.0 : -1.0) * g.xperiod;
  if (g.yper && abs_greater(vy, g.hybits)) vy -= (vy > 0 ? 1.0 : -1.0) * g.yperiod;
}

// Shared-memory bytes of a block whose polygons have `cap` edge slots.
constexpr size_t clip_smem(int cap) {
  return (size_t)cap * CLIP_TPB * (4 * sizeof(double) + sizeof(int) + 4 * sizeof(float));
}

// A polygon of the first pass whose new edge found no free slot, captured at
// that point: its other edges (final for this clip), the new edge's points,
// and where the candidate search stands.  The second pass appends the edge
// in its larger slots and continues the search, so the polygon is computed
// exactly as in one pass with LV_MAX_EDGES slots.  nclips: the clips of the
// first pass, so that the second pass records the polygon's whole count.
struct ClipResume {
  int i, ne, label, pn, s, se, chain_ok, nclips;
  double xx, xy, yx, yy;
  double v1x[ME_SMALL], v1y[ME_SMALL], v2x[ME_SMALL], v2y[ME_SMALL];
  int lab[ME_SMALL];
};

// One polygon per thread (i, active): the whole warp takes part, so threads
// without a polygon pass active = false.  With `save` (the first pass, CAP
// slots), a polygon whose new edge finds no free slot is captured into
// save[atomicAdd(save_n, 1)] and not written; with `resume` (the second
// pass) the polygon continues from such a capture.  Without `save`, running
// out of slots is the reference's edge overflow error.
template <int CAP>
__device__ void clip_polygon(const GridDev& g, const PathNodeDev* __restrict__ path, const double2* __restrict__ x,
                             int i, bool active, const CellsDev& cl, const MeshDev& m, int* status,
                             ClipResume* save, int* save_n, const ClipResume* resume, int slots = CAP) {
  extern __shared__ double smem[];
  const int t = threadIdx.x;
  Poly P;
  P.v1x = smem;
  P.v1y = P.v1x + CAP * CLIP_TPB;
  P.v2x = P.v1y + CAP * CLIP_TPB;
  P.v2y = P.v2x + CAP * CLIP_TPB;
  P.lab = reinterpret_cast<int*>(P.v2y + CAP * CLIP_TPB);
  P.r1x = reinterpret_cast<float*>(P.lab + CAP * CLIP_TPB);
  P.r1y = P.r1x + CAP * CLIP_TPB;
  P.r2x = P.r1y + CAP * CLIP_TPB;
  P.r2y = P.r2x + CAP * CLIP_TPB;
  P.t = t;
  P.cap_e = slots;  // <= CAP

  double px = 0.0, py = 0.0;
  int ne = 0;
  int pn = -1, s = 0, se = 0;
  bool chain_ok = true;
  int nclips = 0;  // clips of the polygon (the order key of the next remesh)
  if (active && resume) {
    const double2 xi = x[i];
    px = xi.x;
    py = xi.y;
    // the captured edges, then the new edge that had no slot
    ne = resume->ne;
    for (int k = 0; k < ne; ++k) {
      set_v1(P, k, resume->v1x[k], resume->v1y[k], px, py);
      set_v2(P, k, resume->v2x[k], resume->v2y[k], px, py);
      P.lab[P.at(k)] = resume->lab[k];
    }
    append_edge(P, ne, resume->xx, resume->xy, resume->yx, resume->yy, px, py, resume->label);
    pn = resume->pn;
    s = resume->s;
    se = resume->se;
    chain_ok = resume->chain_ok != 0;
    nclips = resume->nclips;
  } else if (active) {
    const double2 xi = x[i];
    px = xi.x;
    py = xi.y;
    // reset! (polygon.jl:37-47): the cropping rectangle, edges B->A, A->D, D->C, C->B
    const double Ax = g.cminx, Ay = g.cminy, Cx = g.cmaxx, Cy = g.cmaxy;
    const double Bx = Cx, By = Ay, Dx = Ax, Dy = Cy;
    set_v1(P, 0, Bx, By, px, py); set_v2(P, 0, Ax, Ay, px, py); P.lab[P.at(0)] = LV_BDARY_DOWN;
    set_v1(P, 1, Ax, Ay, px, py); set_v2(P, 1, Dx, Dy, px, py); P.lab[P.at(1)] = LV_BDARY_LEFT;
    set_v1(P, 2, Dx, Dy, px, py); set_v2(P, 2, Cx, Cy, px, py); P.lab[P.at(2)] = LV_BDARY_UP;
    set_v1(P, 3, Cx, Cy, px, py); set_v2(P, 3, Bx, By, px, py); P.lab[P.at(3)] = LV_BDARY_RIGHT;
    ne = 4;
  }
  int flag = 0;
  bool done = !active;
  long long k1 = 0, k2 = 0;
  if (active) {
    const double f1 = floor(div_rcp(px - g.ox, g.h, g.rh)), f2 = floor(div_rcp(py - g.oy, g.h, g.rh));
    if (!(fabs(f1) < 1e15) || !(fabs(f2) < 1e15)) {
      flag = LV_FLAG_NONFINITE;
      done = true;
    } else {
      k1 = (long long)f1 + 1;
      k2 = (long long)f2 + 1;
    }
  }
  // the seed's float offset from its cell's lower corner, and the current
  // path node's cell offset (di1 h, di2 h) in float
  float xo = 0.0f, yo = 0.0f, dhx = 0.0f, dhy = 0.0f;
  if (active && !done) {
    xo = (float)(px - (g.ox + (double)(k1 - 1) * g.h));
    yo = (float)(py - (g.oy + (double)(k2 - 1) * g.h));
    if (pn >= 0 && pn < g.npath) {  // a resumed search: the node it stands in
      const PathNodeDev nd = path[pn];
      dhx = (float)nd.di1 * g.h32;
      dhy = (float)nd.di2 * g.h32;
    }
  }
  // The float offsets of the polygon's vertices (v1 of each edge) in
  // registers for the candidate tests, refreshed after each clip; slots past
  // ne hold the seed (0, 0), which lies inside every half-plane (and adds 0
  // to the influence bound).
  float vrx[CAP], vry[CAP];
  auto cache_poly = [&]() {
#pragma unroll
    for (int k = 0; k < CAP; ++k) {
      const bool in = k < ne;
      vrx[k] = in ? P.r1x[P.at(k)] : 0.0f;
      vry[k] = in ? P.r1y[P.at(k)] : 0.0f;
    }
  };
  // float upper bound of the influence radius prr = max 4 |v1 - x|^2
  auto prr_cached = [&]() -> float {
    float m = 0.0f;
#pragma unroll
    for (int k = 0; k < CAP; ++k) m = fmaxf(m, d2_up(vrx[k], vry[k]));
    return m;
  };
  if (active) cache_poly();
  float prr_up = active ? prr_cached() : 0.0f;
  bool saved = false;
  // whether candidate j (float offset q from its cell's corner) may cut the
  // current polygon; false only when provably not: farther than the
  // influence radius, or every vertex strictly inside the half-plane by more
  // than the rounding margin (the candidate's float offset from the seed
  // carries an absolute error <= g.delta32 per component)
  auto may_cut = [&](int j, float2 q) -> bool {
    if (j == i) return false;  // y == x exactly: get_arrow(x, x) = 0
    if (isnan(q.x)) return true;  // a periodic image: the FP64 clip decides
    const float dx = (q.x - xo) + dhx, dy = (q.y - yo) + dhy;
    const float d2 = dx * dx + dy * dy;
    const float dd = sqrtf(d2);
    const float lo = d2 * (1.0f - 1e-6f) - 4.0f * g.delta32 * dd - 4.0f * g.delta32 * g.delta32;
    if (lo > prr_up * (1.0f + 1e-6f)) return false;  // farther than the influence radius
    if (!chain_ok) return true;
    const float D = dd + 2.0f * g.delta32;
    const float R = 0.5f * sqrtf(prr_up) * 1.0001f;
    const float margin = 2.0f * g.delta32 * (R + 2.0f * D) + 4e-6f * (D * R + D * D) + 4e-15f * D * g.bigm + 1e-14f;
    float fm = 0.0f;  // the seed's value; every vertex's below
#pragma unroll
    for (int k = 0; k < CAP; ++k) fm = fmaxf(fm, __fmaf_rn(dx, vrx[k], dy * vry[k]));
    return !(fm - 0.5f * d2 < -margin);
  };
  // voronoigrid.jl:53-81, in rounds.  Between two clips a lane scans its
  // candidates in groups of up to CLIP_GROUP items of one cell, whose loads
  // are issued together (the scan is bound by the latency of these loads).
  constexpr int CLIP_GROUP = 4;
  while (true) {
    bool have = false;
    int cj = 0;
    while (!done && !have) {
      if (s >= se) {
        ++pn;
        if (pn >= g.npath) {
          done = true;
          break;
        }
        const PathNodeDev nd = path[pn];
        if (nd.rrf > prr_up) {  // prr_up >= prr: never earlier than the reference
          done = true;
          break;
        }
        if (nd.beyond) {
          // the reference stops here if rr > prr, and throws otherwise
          if (!(nd.rr > influence_rr_exact(P, ne, px, py))) flag = LV_FLAG_MESH_DESTROYED;
          done = true;
          break;
        }
        dhx = (float)nd.di1 * g.h32;
        dhy = (float)nd.di2 * g.h32;
        const long long c1 = k1 + nd.di1, c2 = k2 + nd.di2;
        if (c1 < 1 || c1 > g.n1 || c2 < 1 || c2 > g.n2) {
          s = se = 0;
          continue;
        }
        const int cell = (int)((c1 - 1) + (long long)g.n1 * (c2 - 1));
        // (clamped: a cell list that overflowed is reported by the binning)
        se = min(cl.cstart[cell + 1], cl.item_cap);
        s = min(cl.cstart[cell], se);
        if (s >= se) continue;
      }
      const int cnt = min(CLIP_GROUP, se - s);
      int jj[CLIP_GROUP];
      float2 qq[CLIP_GROUP];
#pragma unroll
      for (int u = 0; u < CLIP_GROUP; ++u) {
        const int idx = s + min(u, cnt - 1);
        jj[u] = cl.citem[idx];
        qq[u] = cl.cpos[idx];
      }
      int adv = cnt;
#pragma unroll
      for (int u = 0; u < CLIP_GROUP; ++u)
        if (!have && u < cnt && may_cut(jj[u], qq[u])) {
          have = true;
          cj = jj[u];
          adv = u + 1;
        }
      s += adv;
    }
    if (!__any_sync(0xffffffffu, have)) break;
    nclips += have ? 1 : 0;
    if (have) {
      const double2 xq = x[cj];
      double vx, vy;
      get_arrow(g, xq.x, xq.y, px, py, vx, vy);
      const double yx = px + vx, yy = py + vy;
      int r = 2;
      PendingEdge pend;
      if (chain_ok) r = clip_fast(P, ne, px, py, yx, yy, cj, g.bigm, pend);
      if (r == 2) {
        int nev = 0;
        r = clip_exact(P, ne, px, py, yx, yy, cj, nev, pend);
        // (an edge without a slot counts as added)
        if (nev != 0 && !(r != 0 && nev == 2)) chain_ok = false;
      }
      if (r < 0) {
        if (save) {
          ClipResume& c = save[atomicAdd(save_n, 1)];
          c.i = i;
          c.ne = ne;
          c.label = cj;
          c.pn = pn;
          c.s = s;
          c.se = se;
          c.chain_ok = chain_ok ? 1 : 0;
          c.nclips = nclips;
          c.xx = pend.xx;
          c.xy = pend.xy;
          c.yx = pend.yx;
          c.yy = pend.yy;
          for (int k = 0; k < ne; ++k) {
            const int a = P.at(k);
            c.v1x[k] = P.v1x[a];
            c.v1y[k] = P.v1y[a];
            c.v2x[k] = P.v2x[a];
            c.v2y[k] = P.v2y[a];
            c.lab[k] = P.lab[a];
          }
          saved = true;
        } else {
          flag = LV_FLAG_EDGE_OVERFLOW;
        }
        done = true;
      }
      cache_poly();
      prr_up = prr_cached();
    }
  }
  // a polygon captured for the second pass is not written here
  const bool emit = active && !saved;
  if (emit && flag) atomicOr(status, flag);

  // sort_edges! (IO.jl:35-48)
  const int ne_own = emit ? ne : 0;
  for (int a = 0; a < ne_own; ++a) {
    const double lx = P.v2x[P.at(a)], ly = P.v2y[P.at(a)];
    for (int b = a + 1; b < ne_own; ++b) {
      if (same_value(lx, P.v1x[P.at(b)]) && same_value(ly, P.v1y[P.at(b)])) {
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

  // area (polygon.jl:114-121), centroid (polygon.jl:210-219), faces.  The
  // per-edge work of the warp's polygons is one flat list of (polygon, edge)
  // pairs, 32 per round, so every lane has an edge in every round instead of
  // idling once its own polygon is done.  An edge's terms of the sums go back
  // into its slot and each lane then adds its own polygon's terms in edge
  // order (both sums of the triangle areas run over the same terms in the
  // same order, so one accumulator serves both).  Face f of a polygon is its
  // f-th edge with a neighbour label.  The face lengths are computed on demand.
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wbase = threadIdx.x - lane;
  unsigned fmask = 0u;  // edges with a neighbour (at most LV_MAX_EDGES bits)
  for (int k = 0; k < ne_own; ++k)
    if (P.lab[P.at(k)] >= 0) fmask |= 1u << k;
  int incl = ne_own;  // inclusive prefix of the edge counts over the warp
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += t;
  }
  const int total = __shfl_sync(FULL, incl, 31);
  const int cap = m.cap;
  for (int q0 = 0; q0 < total; q0 += 32) {
    const int q = q0 + lane;
    // the owner lane: the first whose inclusive prefix exceeds q
    int lo = 0, hi = 31;
#pragma unroll
    for (int st = 0; st < 5; ++st) {
      const int mid = (lo + hi) >> 1;
      if (__shfl_sync(FULL, incl, mid) > q) hi = mid;
      else lo = mid + 1;
    }
    const int t = min(lo, 31);
    const int k = q - (__shfl_sync(FULL, incl, t) - __shfl_sync(FULL, ne_own, t));
    const double tpx = __shfl_sync(FULL, px, t), tpy = __shfl_sync(FULL, py, t);
    const int ti = __shfl_sync(FULL, i, t);
    const unsigned tfm = __shfl_sync(FULL, fmask, t);
    if (q < total) {
      const int a = k * CLIP_TPB + wbase + t;
      const double v1x = P.v1x[a], v1y = P.v1y[a], v2x = P.v2x[a], v2y = P.v2y[a];
      const int lab = P.lab[a];
      const double ax = v1x - tpx, ay = v1y - tpy, bx = v2x - tpx, by = v2y - tpy;
      const double dA = 0.5 * fabs(ax * by - ay * bx);
      const double sx = (tpx + v1x) + v2x, sy = (tpy + v1y) + v2y;
      P.v1x[a] = dA;
      P.v1y[a] = div3(dA * sx);
      P.v2x[a] = div3(dA * sy);
      m.ev1[(size_t)k * cap + ti] = make_double2(v1x, v1y);
      m.ev2[(size_t)k * cap + ti] = make_double2(v2x, v2y);
      m.elab[(size_t)k * cap + ti] = lab;
      if (lab >= 0) {
        const double2 xq = x[lab];
        double vx, vy;
        get_arrow(g, xq.x, xq.y, tpx, tpy, vx, vy);
        const double yx = tpx + vx, yy = tpy + vy;
        const double lx = v1x - v2x, ly = v1y - v2y;
        const double l2 = lx * lx + ly * ly;
        const double rx = tpx - yx, ry = tpy - yy;
        const double r2 = rx * rx + ry * ry;
        const size_t f = (size_t)__popc(tfm & ((1u << k) - 1u)) * cap + ti;
        m.fnbr[f] = lab;
        m.flrr[f] = sqrt(l2 / r2);
        m.fm[f] = make_double2(0.5 * (v1x + v2x), 0.5 * (v1y + v2y));
        m.fy[f] = make_double2(yx, yy);
      }
    }
  }
  __syncwarp();
  if (!emit) return;
  double A = 0.0, cx = 0.0, cy = 0.0;
  for (int k = 0; k < ne; ++k) {
    const int a = P.at(k);
    A += P.v1x[a];
    cx = cx + P.v1y[a];
    cy = cy + P.v2x[a];
  }
  m.nedges[i] = ne;
  m.nclip[i] = (unsigned char)min(nclips, 255);
  m.nfaces[i] = __popc(fmask);
  m.area[i] = A;
  m.centroid[i] = make_double2(cx / A, cy / A);
}

// first pass: every polygon with CAP slots; the ones that need more are
// captured into redo[] (redo_n counts them)
template <int CAP>
__global__ void __launch_bounds__(CLIP_TPB) k_clip(GridDev g, const PathNodeDev* __restrict__ path,
                                                   const double2* __restrict__ x, int n, CellsDev cl, MeshDev m,
                                                   int* status, ClipResume* redo, int* redo_n, int slots) {
  const int t = blockIdx.x * CLIP_TPB + threadIdx.x;
  clip_polygon<CAP>(g, path, x, t < n ? m.cperm[t] : 0, t < n, cl, m, status, redo, redo_n, nullptr, slots);
}

// second pass: the captured polygons, resumed with LV_MAX_EDGES slots.  The
// captures are few, so they are dealt round-robin over all resident blocks
// (capture t * gridDim.x + b to thread t of block b): every SM gets some, and
// the pass lasts about one polygon's remaining clipping instead of a block's
// share.
__global__ void __launch_bounds__(CLIP_TPB) k_clip_redo(GridDev g, const PathNodeDev* __restrict__ path,
                                                        const double2* __restrict__ x, CellsDev cl, MeshDev m,
                                                        int* status, const ClipResume* __restrict__ redo,
                                                        const int* __restrict__ redo_n) {
  const int cnt = *redo_n;
  const int per_round = gridDim.x * CLIP_TPB;
  for (int base = 0; base < cnt; base += per_round) {
    if (base + (int)blockIdx.x >= cnt) break;  // nothing for this block (uniform)
    const int q = base + (int)threadIdx.x * (int)gridDim.x + (int)blockIdx.x;
    const bool on = q < cnt;
    // warps without a polygon skip the call (uniform per warp: q grows with the lane)
    if (__any_sync(0xffffffffu, on))
      clip_polygon<ME>(g, path, x, on ? redo[q].i : 0, on, cl, m, status, nullptr, nullptr, on ? redo + q : nullptr);
    __syncwarp();
  }
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

// A stable counting sort of the rows of each window of WIN rows by a small
// key, clamped to 0..32 (one block per window): lanes of a warp with the same key rank
// themselves by __match_any_sync, and the counts of each warp and bucket
// give every bucket's and warp's offset.  The face kernels' row order
// (MeshDev::rperm, by face count) and the clipping's polygon order
// (MeshDev::cperm, by the previous remesh's clip count).
constexpr int RP_BUCKETS = 34;  // keys 0..32, then rows past n
// windows of the clipping's order (256: 24.8, 512: 24.6, 1024: 24.3 ms per
// step of clipping at 4M)
constexpr int CLIP_ORDER_WINDOW = 1024;
template <typename K, int WIN>
__global__ void __launch_bounds__(WIN) k_window_order(const K* __restrict__ key, int n, int* perm) {
  constexpr int NW = WIN / 32;
  __shared__ int wc[NW][RP_BUCKETS], wo[NW][RP_BUCKETS];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int i = blockIdx.x * WIN + t;
  for (int k = t; k < NW * RP_BUCKETS; k += WIN) wc[k / RP_BUCKETS][k % RP_BUCKETS] = 0;
  __syncthreads();
  const int b = i < n ? min(max((int)key[i], 0), RP_BUCKETS - 2) : RP_BUCKETS - 1;
  const unsigned same = __match_any_sync(0xffffffffu, b);
  const int rank = __popc(same & ((1u << lane) - 1u));
  if (lane == __ffs(same) - 1) wc[w][b] = __popc(same);
  __syncthreads();
  if (t < RP_BUCKETS) {
    // bucket t: its start over the window, then each warp's offset in it
    int acc = 0;
    for (int q = 0; q < t; ++q)
      for (int v = 0; v < NW; ++v) acc += wc[v][q];
    for (int v = 0; v < NW; ++v) {
      wo[v][t] = acc;
      acc += wc[v][t];
    }
  }
  __syncthreads();
  if (i < n) perm[blockIdx.x * WIN + wo[w][b] + rank] = i;
}

__global__ void k_face_len(MeshDev m, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) lv_face_lengths(m, i);
}

int lv_mesh_captures_count(lv_ctx* c, int* count) {
  int v = 0;
  cudaMemcpyAsync(&v, c->sv.iters + LV_IT_REDO, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (int rc = lv_cuda_check(c, cudaStreamSynchronize(c->stream), "lv_mesh_captures")) return rc;
  *count = v;
  return LV_OK;
}

int lv_mesh_face_len(lv_ctx* c) {
  if (c->flen_valid) return LV_OK;
  k_face_len<<<lv_blocks(c->n, 256), 256, 0, c->stream>>>(c->m, c->n);
  LV_LAUNCH_CHECK(c, "k_face_len");
  c->flen_valid = true;
  return LV_OK;
}

// The clipping kernels' shared memory and carveout on the current device.
int lv_mesh_device_setup() {
  cudaError_t e = cudaFuncSetAttribute(k_clip<ME_SMALL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)clip_smem(ME_SMALL));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_clip<ME_SMALL>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_clip_redo, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_clip_redo, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)clip_smem(ME));
  return e == cudaSuccess ? LV_OK : LV_ERR_CUDA;
}

int lv_mesh_remesh(lv_ctx* c) {
  const int n = c->n;
  if (n <= 0) return lv_fail(c, LV_ERR_NOT_MESHED, "remesh: no particles");
  c->flen_valid = false;
  c->bnd_valid = false;
  cudaStream_t s = c->stream;
  const int nc = c->c.ncells;
  {
  KernelTimer kt(c, LV_KF_BIN);
  // the cell counts are clean when the previous remesh completed its order pass
  if (!c->ccount_clean) cudaMemsetAsync(c->c.ccount, 0, sizeof(int) * nc, s);
  c->ccount_clean = false;
  k_bin_count<<<lv_blocks(n, 256), 256, 0, s>>>(c->g, c->s.x, n, c->cap, c->c.ccount, c->c.bkey, c->status,
                                                  c->sv.iters + LV_IT_REDO);
  LV_LAUNCH_CHECK(c, "k_bin_count");
  int rc = lv_scan_int(c, c->c.ccount, c->c.cstart, nc);
  if (rc) return rc;
  k_bin_scatter<<<lv_blocks(n, 256), 256, 0, s>>>(c->g, n, c->cap, c->c.bkey, c->c.cstart, c->c.citem,
                                                    c->c.item_cap, c->status);
  LV_LAUNCH_CHECK(c, "k_bin_scatter");
  k_bin_order<<<lv_blocks(nc, 256), 256, 0, s>>>(c->g, c->c.bkey, nc, c->c.cstart, c->c.citem, c->c.cpos, c->s.x,
                                                  c->c.item_cap, c->c.ccount);
  LV_LAUNCH_CHECK(c, "k_bin_order");
  c->ccount_clean = true;
  }
  {
    KernelTimer kt(c, LV_KF_CLIP);
    // the captures for the second pass (one per particle at most), then the count
    if (!c->clip_resume) {
      void* p = nullptr;
      if (cudaMalloc(&p, sizeof(ClipResume) * (size_t)c->cap) != cudaSuccess)
        return lv_fail(c, LV_ERR_CUDA, "allocation of the clipping captures failed");
      c->allocs.push_back(p);
      c->clip_resume = p;
    }
    ClipResume* redo = static_cast<ClipResume*>(c->clip_resume);
    int* redo_n = c->sv.iters + LV_IT_REDO;  // zeroed by k_bin_count
    // the first pass's slots: ME_SMALL, or fewer (5..ME_SMALL-1) through
    // LVGPU_CLIP_SLOTS so that tests can drive most polygons through the
    // second pass (the mesh is the same either way)
    int slots = ME_SMALL;
    if (c->clip_slots >= 5 && c->clip_slots < ME_SMALL) slots = c->clip_slots;
    // the polygon order: by the clip counts of the previous remesh (zeros,
    // so the identity, before the first)
    k_window_order<unsigned char, CLIP_ORDER_WINDOW><<<(n + CLIP_ORDER_WINDOW - 1) / CLIP_ORDER_WINDOW,
                                                       CLIP_ORDER_WINDOW, 0, s>>>(c->m.nclip, n, c->m.cperm);
    LV_LAUNCH_CHECK(c, "k_window_order (clips)");
    k_clip<ME_SMALL><<<lv_blocks(n, CLIP_TPB), CLIP_TPB, clip_smem(ME_SMALL), s>>>(c->g, c->path, c->s.x, n, c->c,
                                                                                   c->m, c->status, redo, redo_n, slots);
    LV_LAUNCH_CHECK(c, "k_clip");
    // three 20-slot blocks fit an SM
    k_clip_redo<<<3 * c->num_sms, CLIP_TPB, clip_smem(ME), s>>>(c->g, c->path, c->s.x, c->c, c->m, c->status,
                                                               redo, redo_n);
    LV_LAUNCH_CHECK(c, "k_clip_redo");
    k_window_order<int, LV_RPERM_WINDOW><<<(n + LV_RPERM_WINDOW - 1) / LV_RPERM_WINDOW, LV_RPERM_WINDOW, 0, s>>>(
        c->m.nfaces, n, c->m.rperm);
    LV_LAUNCH_CHECK(c, "k_window_order (faces)");
  }
  c->meshed = true;
  c->op_ready = false;
  return LV_OK;
}
