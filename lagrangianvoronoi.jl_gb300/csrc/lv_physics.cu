// Per-particle physics operators of the time step, one thread per polygon.
//
// Every operator walks the polygon's interior faces in the order of
// `neighbors(p, grid)` (src/iterators.jl:23-33) from the slot-major face
// arrays written by the clipping kernel (neighbour index, lr_ratio, midpoint,
// neighbour position y, edge length), so no geometry is recomputed here.
// Two-pass operators of the reference (a read phase and a write phase over
// all polygons) are two kernel launches.
//
// Compiled with --fmad=false: expressions keep the reference's evaluation
// order and rounding, so results are bit-identical to a sequential FP64
// evaluation of the same formulas in the same face order.
#include <math.h>

#include <algorithm>

#include "lv_internal.cuh"

namespace {

constexpr int TPB = 256;

// Face loops load FB faces at a time (slot indexes clamped to the last face)
// so that the loads of a particle's faces overlap instead of forming one
// chain of dependent round trips; the arithmetic then runs over the faces
// in order, as before.
constexpr int FB = 8;
__device__ __forceinline__ size_t face_slot(int k, int nf, int cap, int i) {
  return (size_t)(k < nf ? k : nf - 1) * cap + i;
}

__device__ __forceinline__ double jmax(double a, double b) { return (b > a) ? b : a; }
__device__ __forceinline__ double jmin(double a, double b) { return (b < a) ? b : a; }
// a wall velocity pair (x, y of two labels), passed to kernels by value
struct Wall2 {
  double x, y, z, w;
};

// ------------------------------------------------------------------- EOS

// ideal_eos! (pressure.jl:49-55), stiffened_eos! (pressure.jl:64-70),
// find_rho! (pressure.jl:36-40).  kind 0: ideal (p = Pmin), 1: stiffened
// (p = P0), 2: density only.
__global__ void k_eos(StateDev s, MeshDev m, int n, int kind, double gamma, double pp) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double rho = s.mass[i] / m.area[i];
  s.rho[i] = rho;
  if (kind == 2) return;
  double2 v = s.v[i];
  double eint = s.e[i] - 0.5 * (v.x * v.x + v.y * v.y);
  double P = (gamma - 1.0) * rho * eint;
  s.P[i] = P;
  if (kind == 0)
    s.c2[i] = gamma * jmax(P, pp) / rho;
  else
    s.c2[i] = gamma * (P + pp) / rho;
}

// gravity_step! (pressure.jl:77-82)
__global__ void k_gravity(StateDev s, int n, double gx, double gy, double dt) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double2 v = s.v[i];
  s.v[i] = make_double2(v.x + dt * gx, v.y + dt * gy);
}

// ------------------------------------------------------------ pressure step

// pressure_step! (pressure.jl:10-25), velocity pass.
__global__ void k_pstep_v(StateDev s, MeshDev m, int n, double dt) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = face_row(m, t);
  const int cap = m.cap, nf = m.nfaces[i];
  const double2 xi = s.x[i];
  const double Pi = s.P[i], mi = s.mass[i];
  double2 vi = s.v[i];
  for (int k0 = 0; k0 < nf; k0 += FB) {
    int j[FB];
    double lrr[FB], pj[FB];
    double2 mm[FB];
#pragma unroll
    for (int u = 0; u < FB; ++u) {
      const size_t f = face_slot(k0 + u, nf, cap, i);
      j[u] = ld_nc(m.fnbr + f);
      lrr[u] = ld_nc(m.flrr + f);
      mm[u] = ld_nc(m.fm + f);
    }
#pragma unroll
    for (int u = 0; u < FB; ++u) pj[u] = ld_nc(s.P + j[u]);
#pragma unroll
    for (int u = 0; u < FB; ++u) {
      if (k0 + u >= nf) break;
      const double c = dt / mi * lrr[u] * (Pi - pj[u]);
      vi.x = vi.x + c * (mm[u].x - xi.x);
      vi.y = vi.y + c * (mm[u].y - xi.y);
    }
  }
  s.v[i] = vi;
}

// pressure_step! energy pass (uses the updated velocities).
__global__ void __launch_bounds__(TPB, 2) k_pstep_e(StateDev s, MeshDev m, int n, double dt) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = face_row(m, t);
  const int cap = m.cap, nf = m.nfaces[i];
  const double2 xi = s.x[i];
  const double Pi = s.P[i], mi = s.mass[i];
  const double rmi = 1.0 / mi;  // the per-face divisions by mi through div_rcp
  const double2 vi = s.v[i];
  const double2 Pv = make_double2(Pi * vi.x, Pi * vi.y);
  double ei = s.e[i];
  constexpr int B = FB / 2;
  for (int k0 = 0; k0 < nf; k0 += B) {
    int j[B];
    double lrr[B], Pj[B];
    double2 mm[B], y[B], vj[B];
#pragma unroll
    for (int u = 0; u < B; ++u) {
      const size_t f = face_slot(k0 + u, nf, cap, i);
      j[u] = ld_nc(m.fnbr + f);
      lrr[u] = ld_nc(m.flrr + f);
      mm[u] = ld_nc(m.fm + f);
      y[u] = ld_nc(m.fy + f);
    }
#pragma unroll
    for (int u = 0; u < B; ++u) {
      Pj[u] = ld_nc(s.P + j[u]);
      vj[u] = ld_nc(s.v + j[u]);
    }
#pragma unroll
    for (int u = 0; u < B; ++u) {
      if (k0 + u >= nf) break;
      const double2 Pvj = make_double2(Pj[u] * vj[u].x, Pj[u] * vj[u].y);
      const double a = (mm[u].x - xi.x) * Pv.x + (mm[u].y - xi.y) * Pv.y;
      const double b = (mm[u].x - y[u].x) * Pvj.x + (mm[u].y - y[u].y) * Pvj.y;
      ei -= div_rcp(dt * lrr[u], mi, rmi) * (a - b);
    }
  }
  s.e[i] = ei;
}

// ------------------------------------------------------------- RHS refresh

// refresh!(solver, dt, gp_step, vbc) (pressure.jl:162-201): b, the warm
// start P and the pressure gradient GP.  It splits into the terms that stay fixed over
// the fixed-point sweeps of find_pressure! (v, the mesh and the walls do not
// change between them) and those that follow P.  k_rhs_prep evaluates the
// fixed ones once per find_pressure! with the reference's expressions:
//   tf  = (lrr/dt) dot(v_i - v_j, m - y)        per face
//   dmz = m - midpoint(x_i, y)                  per face (explicit Laplacian)
//   te  = dot(dS, vbc - v_i)/dt                 per boundary edge
// and k_rhs / k_rhs_gp subtract or add them in the reference's order, so b and
// GP are bit-identical to evaluating refresh! in full every sweep.
// Boundary velocities come from the label table, or per boundary edge (bvel,
// the edges of polygon i from boff[i] on, in its edge order) when bvel is set.
__global__ void __launch_bounds__(TPB, 2) k_rhs_prep(StateDev s, MeshDev m, SolverDev sv, int n, double dt, Wall2 vbc_ud,
                                                     Wall2 vbc_rl, const double2* __restrict__ bvel,
                                                     const int* __restrict__ boff) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = face_row(m, t);
  const int cap = m.cap, nf = m.nfaces[i], ne = m.nedges[i];
  const double2 xi = s.x[i];
  const double2 vi = s.v[i];
  // the fixed factors of k_rhs: the divisor of the first term with its
  // reciprocal, and the reciprocal of the mass (divisions by div_rcp)
  const double den = s.rho[i] * s.c2[i] * (dt * dt);
  sv.rhs_den[i] = den;
  sv.rhs_rden[i] = 1.0 / den;
  sv.rhs_rm[i] = 1.0 / s.mass[i];
  constexpr int B = FB / 2;
  for (int k0 = 0; k0 < nf; k0 += B) {
    int j[B];
    double lrr[B];
    double2 mm[B], y[B], vj[B];
#pragma unroll
    for (int u = 0; u < B; ++u) {
      const size_t f = face_slot(k0 + u, nf, cap, i);
      j[u] = ld_nc(m.fnbr + f);
      lrr[u] = ld_nc(m.flrr + f);
      mm[u] = ld_nc(m.fm + f);
      y[u] = ld_nc(m.fy + f);
    }
#pragma unroll
    for (int u = 0; u < B; ++u) vj[u] = ld_nc(s.v + j[u]);
#pragma unroll
    for (int u = 0; u < B; ++u) {
      if (k0 + u >= nf) break;
      const size_t f = (size_t)(k0 + u) * cap + i;
      sv.rhs_tf[f] = (lrr[u] / dt) * ((vi.x - vj[u].x) * (mm[u].x - y[u].x) + (vi.y - vj[u].y) * (mm[u].y - y[u].y));
      const double zx = 0.5 * (xi.x + y[u].x), zy = 0.5 * (xi.y + y[u].y);
      sv.rhs_dmz[f] = make_double2(mm[u].x - zx, mm[u].y - zy);
      sv.rhs_dm[f] = make_double2(mm[u].x - xi.x, mm[u].y - xi.y);
    }
  }
  if (nf < ne) {
    int jb = bvel ? boff[i] : 0;
    for (int k = 0; k < ne; ++k) {
      const size_t f = (size_t)k * cap + i;
      const int lab = m.elab[f];
      if (lab >= 0) continue;
      const double2 a = m.ev1[f], b = m.ev2[f];
      const double dSx = a.y - b.y, dSy = b.x - a.x;
      double wx, wy;
      if (bvel) {
        const double2 wv = bvel[jb++];
        wx = wv.x;
        wy = wv.y;
      } else {
        switch (lab) {
          case LV_BDARY_UP: wx = vbc_ud.x; wy = vbc_ud.y; break;
          case LV_BDARY_RIGHT: wx = vbc_rl.x; wy = vbc_rl.y; break;
          case LV_BDARY_DOWN: wx = vbc_ud.z; wy = vbc_ud.w; break;
          default: wx = vbc_rl.z; wy = vbc_rl.w; break;
        }
      }
      sv.rhs_te[f] = (dSx * (wx - vi.x) + dSy * (wy - vi.y)) / dt;
    }
  }
}

// refresh! first loop (pressure.jl:167-186) with the fixed terms of k_rhs_prep.
// guess 1: also d1 = P - pprev in FP32 for the sweep's initial guess; guess 2
// (sweep 1): the sums of the initial guess with the residual b - A P and the
// previous call's change D (lv_sweep_sums; all threads of the block take
// part, so rows past n do not return early).
// (four blocks per SM: 64 registers with a few spills, 0.17 ms per step faster at 4M than 80 at three)
__global__ void __launch_bounds__(TPB, 4) k_rhs(StateDev s, MeshDev m, SolverDev sv, int n, double dt, int guess, const float* D) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const bool on = t < n;
  const int i = on ? face_row(m, t) : t;
  double bi = 0.0, Pi = 0.0;
  if (on) {
    const int cap = m.cap, nf = m.nfaces[i], ne = m.nedges[i];
    Pi = s.P[i];
    if (guess == 1) sv.sgd32[i] = (float)(Pi - sv.pprev[i]);
    // area Pi / (rho c2 dt^2), with the divisor and its reciprocal from k_rhs_prep
    bi = div_rcp(m.area[i] * Pi, sv.rhs_den[i], sv.rhs_rden[i]);
    double gpx = 0.0, gpy = 0.0;
    for (int k0 = 0; k0 < nf; k0 += FB) {
      int j[FB];
      double lrr[FB], tf[FB], pj[FB];
      double2 dm[FB];  // m - x_i
#pragma unroll
      for (int u = 0; u < FB; ++u) {
        const size_t f = face_slot(k0 + u, nf, cap, i);
        j[u] = ld_nc(m.fnbr + f);
        lrr[u] = ld_nc(m.flrr + f);
        dm[u] = ld_nc(sv.rhs_dm + f);
        tf[u] = ld_nc(sv.rhs_tf + f);
      }
#pragma unroll
      for (int u = 0; u < FB; ++u) pj[u] = ld_nc(s.P + j[u]);
#pragma unroll
      for (int u = 0; u < FB; ++u) {
        if (k0 + u >= nf) break;
        bi -= tf[u];
        const double c = lrr[u] * (Pi - pj[u]);
        gpx = gpx - c * dm[u].x;
        gpy = gpy - c * dm[u].y;
      }
    }
    if (nf < ne) {
      for (int k = 0; k < ne; ++k) {
        const size_t f = (size_t)k * cap + i;
        if (m.elab[f] < 0) bi -= sv.rhs_te[f];
      }
    }
    sv.b[i] = bi;
    sv.xs[i] = Pi;
    const double mi = s.mass[i], rm = sv.rhs_rm[i];
    s.GP[i] = make_double2(div_rcp(gpx, mi, rm), div_rcp(gpy, mi, rm));
  }
  if (guess == 2) {
    double res = 0.0;
    if (on) {
      // b - A P with the operator's difference form
      double ap = sv.diag[i] * Pi;
      const int e0 = sv.rowptr[i], e1 = sv.rowptr[i + 1];
      for (int b0 = e0; b0 < e1; b0 += FB) {
        int j[FB];
        double w[FB], pj[FB];
#pragma unroll
        for (int u = 0; u < FB; ++u) {
          const int e = min(b0 + u, e1 - 1);
          j[u] = ld_nc(sv.col + e);
          w[u] = ld_nc(sv.w + e);
        }
#pragma unroll
        for (int u = 0; u < FB; ++u) pj[u] = ld_nc(s.P + j[u]);
#pragma unroll
        for (int u = 0; u < FB; ++u) {
          if (b0 + u >= e1) break;
          ap += w[u] * (Pi - pj[u]);
        }
      }
      res = bi - ap;
    }
    lv_sweep_sums(sv, i, on, res, 0.0, D, false, true, n);
  }
}

// refresh! second loop (pressure.jl:189-201): explicit part of the Laplacian.
// guess != 0: then the sums of the sweep's initial guess with the directions
// d1 and D (nullptr: none) and the residual b_k - b_{k-1} (lv_sweep_sums;
// all threads of the block take part, so rows past n do not return early).
__global__ void k_rhs_gp(StateDev s, MeshDev m, SolverDev sv, int n, int guess, const float* D) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const bool on = t < n;
  const int i = on ? face_row(m, t) : t;
  double bi = 0.0;
  if (on) {
    const int cap = m.cap, nf = m.nfaces[i];
    const double2 gi = s.GP[i];
    bi = sv.b[i];
    for (int k0 = 0; k0 < nf; k0 += FB) {
      int j[FB];
      double lrr[FB];
      double2 dmz[FB], gj[FB];
#pragma unroll
      for (int u = 0; u < FB; ++u) {
        const size_t f = face_slot(k0 + u, nf, cap, i);
        j[u] = ld_nc(m.fnbr + f);
        lrr[u] = ld_nc(m.flrr + f);
        dmz[u] = ld_nc(sv.rhs_dmz + f);
      }
#pragma unroll
      for (int u = 0; u < FB; ++u) gj[u] = ld_nc(s.GP + j[u]);
#pragma unroll
      for (int u = 0; u < FB; ++u) {
        if (k0 + u >= nf) break;
        bi += lrr[u] * ((gi.x - gj[u].x) * dmz[u].x + (gi.y - gj[u].y) * dmz[u].y);
      }
    }
    sv.b[i] = bi;
  }
  if (guess) {
    const double res = on ? bi - sv.bprev[i] : 0.0;
    const double d1 = on ? s.P[i] - sv.pprev[i] : 0.0;
    lv_sweep_sums(sv, i, on, res, d1, D, true, D != nullptr, n);
  }
}

// ---------------------------------------------------------- viscosity, D

// find_D! (diffusion.jl:8-19)
__global__ void k_find_D(StateDev s, MeshDev m, int n) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = face_row(m, t);
  const int cap = m.cap, nf = m.nfaces[i];
  const double2 vi = s.v[i];
  double d11 = 0.0, d21 = 0.0, d12 = 0.0, d22 = 0.0;
  for (int k0 = 0; k0 < nf; k0 += FB) {
    int j[FB];
    double lrr[FB];
    double2 mm[FB], y[FB], vj[FB];
#pragma unroll
    for (int u = 0; u < FB; ++u) {
      const size_t f = face_slot(k0 + u, nf, cap, i);
      j[u] = ld_nc(m.fnbr + f);
      lrr[u] = ld_nc(m.flrr + f);
      mm[u] = ld_nc(m.fm + f);
      y[u] = ld_nc(m.fy + f);
    }
#pragma unroll
    for (int u = 0; u < FB; ++u) vj[u] = ld_nc(s.v + j[u]);
#pragma unroll
    for (int u = 0; u < FB; ++u) {
      if (k0 + u >= nf) break;
      const double ax = vi.x - vj[u].x, ay = vi.y - vj[u].y, bx = mm[u].x - y[u].x, by = mm[u].y - y[u].y;
      d11 += lrr[u] * (ax * bx);
      d21 += lrr[u] * (ay * bx);
      d12 += lrr[u] * (ax * by);
      d22 += lrr[u] * (ay * by);
    }
  }
  const double A = m.area[i];
  d11 = d11 / A;
  d21 = d21 / A;
  d12 = d12 / A;
  d22 = d22 / A;
  s.Da[i] = make_double2(0.5 * (d11 + d11), 0.5 * (d21 + d12));
  s.Db[i] = make_double2(0.5 * (d12 + d21), 0.5 * (d22 + d22));
}

// getS (diffusion.jl:22-29): viscous stress, stored in GP-sized scratch as
// two double2 per particle (S11,S21) and (S12,S22).
__global__ void k_stress(StateDev s, int n, double avdr, double2* Sa, double2* Sb) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 a = s.Da[i], b = s.Db[i];
  const double divv = a.x + b.y;
  double mu = s.mu[i];
  if (divv < 0.0) mu -= divv * s.rho[i] * (avdr * avdr);
  const double c = 2.0 * mu;
  Sa[i] = make_double2(c * (a.x - divv / 3.0), c * a.y);
  Sb[i] = make_double2(c * b.x, c * (b.y - divv / 3.0));
}

// viscous_step! velocity pass (diffusion.jl:41-46)
__global__ void __launch_bounds__(TPB, 2) k_visc_v(StateDev s, MeshDev m, int n, double dt, const double2* __restrict__ Sa,
                         const double2* __restrict__ Sb) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = face_row(m, t);
  const int cap = m.cap, nf = m.nfaces[i];
  const double2 xi = s.x[i];
  const double mi = s.mass[i];
  const double rmi = 1.0 / mi;  // the per-face divisions by mi through div_rcp
  const double2 sa = Sa[i], sb = Sb[i];
  double2 vi = s.v[i];
  constexpr int B = FB / 2;
  for (int k0 = 0; k0 < nf; k0 += B) {
    int j[B];
    double lrr[B];
    double2 mm[B], qa[B], qb[B];
#pragma unroll
    for (int u = 0; u < B; ++u) {
      const size_t f = face_slot(k0 + u, nf, cap, i);
      j[u] = ld_nc(m.fnbr + f);
      lrr[u] = ld_nc(m.flrr + f);
      mm[u] = ld_nc(m.fm + f);
    }
#pragma unroll
    for (int u = 0; u < B; ++u) {
      qa[u] = ld_nc(Sa + j[u]);
      qb[u] = ld_nc(Sb + j[u]);
    }
#pragma unroll
    for (int u = 0; u < B; ++u) {
      if (k0 + u >= nf) break;
      const double c = div_rcp(dt * lrr[u], mi, rmi);
      const double M11 = c * (sa.x - qa[u].x), M21 = c * (sa.y - qa[u].y), M12 = c * (sb.x - qb[u].x),
                   M22 = c * (sb.y - qb[u].y);
      const double dx = mm[u].x - xi.x, dy = mm[u].y - xi.y;
      vi.x = vi.x - (M11 * dx + M12 * dy);
      vi.y = vi.y - (M21 * dx + M22 * dy);
    }
  }
  s.v[i] = vi;
}

// viscous_step! energy pass (diffusion.jl:47-52)
__global__ void __launch_bounds__(TPB, 2) k_visc_e(StateDev s, MeshDev m, int n, double dt, const double2* __restrict__ Sa,
                         const double2* __restrict__ Sb) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = face_row(m, t);
  const int cap = m.cap, nf = m.nfaces[i];
  const double2 xi = s.x[i];
  const double mi = s.mass[i];
  const double rmi = 1.0 / mi;  // the per-face divisions by mi through div_rcp
  const double2 sa = Sa[i], sb = Sb[i];
  const double2 vi = s.v[i];
  const double Svx = sa.x * vi.x + sb.x * vi.y, Svy = sa.y * vi.x + sb.y * vi.y;
  double ei = s.e[i];
  constexpr int B = FB / 2;
  for (int k0 = 0; k0 < nf; k0 += B) {
    int j[B];
    double lrr[B];
    double2 mm[B], y[B], qa[B], qb[B], vj[B];
#pragma unroll
    for (int u = 0; u < B; ++u) {
      const size_t f = face_slot(k0 + u, nf, cap, i);
      j[u] = ld_nc(m.fnbr + f);
      lrr[u] = ld_nc(m.flrr + f);
      mm[u] = ld_nc(m.fm + f);
      y[u] = ld_nc(m.fy + f);
    }
#pragma unroll
    for (int u = 0; u < B; ++u) {
      qa[u] = ld_nc(Sa + j[u]);
      qb[u] = ld_nc(Sb + j[u]);
      vj[u] = ld_nc(s.v + j[u]);
    }
#pragma unroll
    for (int u = 0; u < B; ++u) {
      if (k0 + u >= nf) break;
      const double Sqx = qa[u].x * vj[u].x + qb[u].x * vj[u].y, Sqy = qa[u].y * vj[u].x + qb[u].y * vj[u].y;
      const double a = (mm[u].x - xi.x) * Svx + (mm[u].y - xi.y) * Svy;
      const double b = (mm[u].x - y[u].x) * Sqx + (mm[u].y - y[u].y) * Sqy;
      ei += div_rcp(dt * lrr[u], mi, rmi) * (a - b);
    }
  }
  s.e[i] = ei;
}

// bdary_friction! (diffusion.jl:64-79): the wall velocity from the label
// table, or per boundary edge (bvel from boff[i], as in k_rhs_prep) with the
// edges whose act is 0 skipped (charfun; act may be null).
__global__ void k_friction(StateDev s, MeshDev m, int n, double dt, Wall2 w_ud, Wall2 w_rl,
                           const double2* __restrict__ bvel, const int* __restrict__ boff,
                           const unsigned char* __restrict__ act) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = face_row(m, t);
  const int cap = m.cap, nf = m.nfaces[i], ne = m.nedges[i];
  if (nf == ne) {
    // no boundary edge: v = v/1.0 leaves v unchanged
    return;
  }
  const double2 xi = s.x[i];
  const double mu = s.mu[i], mi = s.mass[i];
  double tmp = 1.0;
  double2 vi = s.v[i];
  double ei = s.e[i];
  int jb = bvel ? boff[i] : 0;
  for (int k = 0; k < ne; ++k) {
    const size_t f = (size_t)k * cap + i;
    const int lab = m.elab[f];
    if (lab >= 0) continue;
    const int q = jb++;
    if (bvel && act && !act[q]) continue;  // if !charfun(m) continue end
    const double2 a = m.ev1[f], b = m.ev2[f];
    const double mx = 0.5 * (a.x + b.x), my = 0.5 * (a.y + b.y);
    const double nx0 = a.y - b.y, ny0 = b.x - a.x;
    const double nn = sqrt(nx0 * nx0 + ny0 * ny0);
    const double nx = nx0 / nn, ny = ny0 / nn;
    const double lx = a.x - b.x, ly = a.y - b.y;
    const double len = sqrt(lx * lx + ly * ly);
    const double lrr = len / fabs((mx - xi.x) * nx + (my - xi.y) * ny);
    double wx, wy;
    if (bvel) {
      wx = bvel[q].x;
      wy = bvel[q].y;
    } else {
      switch (lab) {
        case LV_BDARY_UP: wx = w_ud.x; wy = w_ud.y; break;
        case LV_BDARY_RIGHT: wx = w_rl.x; wy = w_rl.y; break;
        case LV_BDARY_DOWN: wx = w_ud.z; wy = w_ud.w; break;
        default: wx = w_rl.z; wy = w_rl.w; break;
      }
    }
    const double fx = mu * lrr * wx / mi, fy = mu * lrr * wy / mi;
    tmp += dt * mu * lrr / mi;
    ei += dt * (fx * vi.x + fy * vi.y);
    vi.x = vi.x + dt * fx;
    vi.y = vi.y + dt * fy;
  }
  s.v[i] = make_double2(vi.x / tmp, vi.y / tmp);
  s.e[i] = ei;
}

// ---------------------------------------------------------- relaxation

// find_dv! (relaxation.jl:10-25)
__global__ void k_find_dv(StateDev s, MeshDev m, int n, double dt, double alpha) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = face_row(m, t);
  const int cap = m.cap, nf = m.nfaces[i];
  const double2 xi = s.x[i];
  const double2 c = m.centroid[i];
  // the extreme distances are the square roots of the extreme squared
  // distances (sqrt is correctly rounded and monotone, and jmax/jmin keep
  // the first of equal values), so two square roots instead of one per face
  double r2max = 0.0, r2min = __longlong_as_double(0x7ff0000000000000LL);
  for (int k0 = 0; k0 < nf; k0 += FB) {
    double2 y[FB];
#pragma unroll
    for (int u = 0; u < FB; ++u) y[u] = ld_nc(m.fy + face_slot(k0 + u, nf, cap, i));
#pragma unroll
    for (int u = 0; u < FB; ++u) {
      if (k0 + u >= nf) break;
      const double dx = xi.x - y[u].x, dy = xi.y - y[u].y;
      const double r2 = dx * dx + dy * dy;
      r2max = jmax(r2max, r2);
      r2min = jmin(r2min, r2);
    }
  }
  const double rmax = sqrt(r2max), rmin = sqrt(r2min);
  const double q = rmin / rmax;
  s.quality[i] = q;
  const double2 a = s.Da[i], b = s.Db[i];
  const double nD = sqrt(a.x * a.x + a.y * a.y + b.x * b.x + b.y * b.y);
  const double lambda = alpha * nD / (q * q);
  const double f = lambda / (1.0 + dt * lambda);
  s.dv[i] = make_double2(f * (c.x - xi.x), f * (c.y - xi.y));
}

// relaxation_step! first loop (relaxation.jl:37-66): conservative remap of
// mass, momentum and energy along dv with the Rusanov flux.
// |dv| of every particle, evaluated once instead of on every face that
// reads it (the same expression, so the same value); lens: also the face
// lengths of the mesh (lv_face_lengths)
__global__ void k_norm_dv(StateDev s, MeshDev m, int n, double* ndv, int lens) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = face_row(m, t);
  const double2 d = s.dv[i];
  ndv[i] = sqrt(d.x * d.x + d.y * d.y);
  if (lens) lv_face_lengths(m, i);
}

// ndv: |dv| of every particle (k_norm_dv), read when rusanov is set
__global__ void __launch_bounds__(TPB, 2) k_relax_flux(StateDev s, MeshDev m, int n, double dt, int rusanov, const double* __restrict__ ndv) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = face_row(m, t);
  const int cap = m.cap, nf = m.nfaces[i];
  const double2 xi = s.x[i];
  const double rp = s.rho[i], ep = s.e[i];
  const double2 vp = s.v[i], dvp = s.dv[i];
  const int php = s.phase[i];
  double mass = s.mass[i];
  double momx = mass * vp.x, momy = mass * vp.y;
  double energy = mass * ep;
  const double ndvp = rusanov ? ndv[i] : 0.0;
  constexpr int B = 2;  // six gathers per face
  for (int k0 = 0; k0 < nf; k0 += B) {
    int jb[B], phb[B];
    double lrrb[B], lb[B], rqb[B], eqb[B], nqb[B];
    double2 mmb[B], yb[B], vqb[B], dvqb[B];
#pragma unroll
    for (int u = 0; u < B; ++u) {
      const size_t f = face_slot(k0 + u, nf, cap, i);
      jb[u] = ld_nc(m.fnbr + f);
      lrrb[u] = ld_nc(m.flrr + f);
      mmb[u] = ld_nc(m.fm + f);
      yb[u] = ld_nc(m.fy + f);
      lb[u] = rusanov ? ld_nc(m.flen + f) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < B; ++u) {
      const int j = jb[u];
      phb[u] = ld_nc(s.phase + j);
      rqb[u] = ld_nc(s.rho + j);
      eqb[u] = ld_nc(s.e + j);
      vqb[u] = ld_nc(s.v + j);
      dvqb[u] = ld_nc(s.dv + j);
      nqb[u] = rusanov ? ld_nc(ndv + j) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < B; ++u) {
      if (k0 + u >= nf) break;
      if (phb[u] != php) continue;
      const double lrr = lrrb[u];
      const double2 mm = mmb[u], y = yb[u];
      const double zx = 0.5 * (xi.x + y.x), zy = 0.5 * (xi.y + y.y);
      const double rq = rqb[u], eq = eqb[u];
      const double2 vq = vqb[u], dvq = dvqb[u];
      const double pqx = xi.x - y.x, pqy = xi.y - y.y;
      const double mzx = mm.x - zx, mzy = mm.y - zy;
      const double pdvpq = dvp.x * pqx + dvp.y * pqy;
      const double qdvpq = dvq.x * pqx + dvq.y * pqy;
      const double pdvmz = dvp.x * mzx + dvp.y * mzy;
      const double qdvmz = dvq.x * mzx + dvq.y * mzy;
      const double kk = dt * lrr;
      mass += kk * ((pdvmz * rp - qdvmz * rq) - 0.5 * (pdvpq * rp + qdvpq * rq));
      const double a1 = pdvmz * rp, a2 = qdvmz * rq, b1 = pdvpq * rp, b2 = qdvpq * rq;
      const double t1x = a1 * vp.x - a2 * vq.x, t1y = a1 * vp.y - a2 * vq.y;
      const double t2x = b1 * vp.x + b2 * vq.x, t2y = b1 * vp.y + b2 * vq.y;
      momx = momx + kk * (t1x - 0.5 * t2x);
      momy = momy + kk * (t1y - 0.5 * t2y);
      energy += kk * ((pdvmz * rp * ep - qdvmz * rq * eq) - 0.5 * (pdvpq * rp * ep + qdvpq * rq * eq));
      if (rusanov) {
        const double ndvq = nqb[u];
        const double a = jmax(ndvp, ndvq);
        const double l = lb[u];
        const double cr = 0.5 * dt * l * a;
        mass += cr * (rq - rp);
        momx = momx + cr * (rq * vq.x - rp * vp.x);
        momy = momy + cr * (rq * vq.y - rp * vp.y);
        energy += cr * (rq * eq - rp * ep);
      }
    }
  }
  s.mass[i] = mass;
  s.mom[i] = make_double2(momx, momy);
  s.energy[i] = energy;
}

// relaxation_step! second loop (relaxation.jl:67-71)
__global__ void k_relax_update(StateDev s, int n, double dt) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double mass = s.mass[i];
  const double2 mom = s.mom[i];
  s.v[i] = make_double2(mom.x / mass, mom.y / mass);
  s.e[i] = s.energy[i] / mass;
  const double2 x = s.x[i], dv = s.dv[i];
  s.x[i] = make_double2(x.x + dt * dv.x, x.y + dt * dv.y);
}

// ----------------------------------------------------------------- move

// least_positive_residue / periodic_wrap (voronoigrid.jl:181-192)
__device__ __forceinline__ double lpr(double x, double d) { return fmod(fmod(x, d) + d, d); }

__device__ __forceinline__ bool try_move(const GridDev& g, double2& x, double2 v, double dt) {
  double nx = x.x + dt * v.x, ny = x.y + dt * v.y;
  const double wx = lpr(nx - g.bminx, g.xperiod) + g.bminx;
  const double wy = lpr(ny - g.bminy, g.yperiod) + g.bminy;
  if (g.xper) nx = nx + (wx - nx);
  if (g.yper) ny = ny + (wy - ny);
  if (g.bminx <= nx && nx <= g.bmaxx && g.bminy <= ny && ny <= g.bmaxy) {
    x = make_double2(nx, ny);
    return true;
  }
  return false;
}

// move! (move.jl:9-21) and try_move! (move.jl:23-33), without the remesh.
__global__ void k_move(GridDev g, StateDev s, MeshDev m, int n, double dt, int* status) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double2 x = s.x[i];
  double2 v = s.v[i];
  if (isnan(v.x) || isnan(v.y)) {
    atomicOr(status, LV_FLAG_NAN_VELOCITY);
    return;
  }
  if (try_move(g, x, v, dt)) {
    s.x[i] = x;
    return;
  }
  const int cap = m.cap, ne = m.nedges[i];
  for (int k = 0; k < ne; ++k) {
    const size_t f = (size_t)k * cap + i;
    if (m.elab[f] >= 0) continue;
    const double2 a = m.ev1[f], b = m.ev2[f];
    const double nx0 = a.y - b.y, ny0 = b.x - a.x;
    const double nn = sqrt(nx0 * nx0 + ny0 * ny0);
    const double nx = nx0 / nn, ny = ny0 / nn;
    const double d = v.x * nx + v.y * ny;
    v.x = v.x - d * nx;
    v.y = v.y - d * ny;
  }
  if (isnan(v.x) || isnan(v.y)) {
    atomicOr(status, LV_FLAG_NAN_VELOCITY);
    return;
  }
  if (!try_move(g, x, v, dt)) {
    v = make_double2(0.0, 0.0);
    try_move(g, x, v, dt);
  }
  s.x[i] = x;
  s.v[i] = v;
}

// ----------------------------------------------------- multiphase projector

// relaxation.jl:157-169: b_i = -sum_{cross-phase faces} lrr (dot(dv_i - dv_j, m - z)
//                                   - 0.5 dot(dv_i + dv_j, x_i - y))
__global__ void k_mp_rhs(StateDev s, MeshDev m, int n, double* b) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = face_row(m, t);
  const int cap = m.cap, nf = m.nfaces[i];
  const double2 xi = s.x[i], dvi = s.dv[i];
  const int ph = s.phase[i];
  double bi = 0.0;
  for (int k = 0; k < nf; ++k) {
    const size_t f = (size_t)k * cap + i;
    const int j = m.fnbr[f];
    if (s.phase[j] == ph) continue;
    const double lrr = m.flrr[f];
    const double2 mm = m.fm[f], y = m.fy[f];
    const double2 dvj = s.dv[j];
    const double zx = 0.5 * (xi.x + y.x), zy = 0.5 * (xi.y + y.y);
    const double a = (dvi.x - dvj.x) * (mm.x - zx) + (dvi.y - dvj.y) * (mm.y - zy);
    const double c = (dvi.x + dvj.x) * (xi.x - y.x) + (dvi.y + dvj.y) * (xi.y - y.y);
    bi -= lrr * (a - 0.5 * c);
  }
  b[i] = bi;
}

// relaxation.jl:92-106: tmp_i = -(1/area) sum lrr (x_i - x_j)(m - x_i)
__global__ void k_mp_apply1(StateDev s, MeshDev m, int n, const double* __restrict__ xin, double2* tmp) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = face_row(m, t);
  const int cap = m.cap, nf = m.nfaces[i];
  const double2 xi = s.x[i];
  const int ph = s.phase[i];
  double tx = 0.0, ty = 0.0;
  const double xv = xin[i];
  for (int k = 0; k < nf; ++k) {
    const size_t f = (size_t)k * cap + i;
    const int j = m.fnbr[f];
    if (s.phase[j] == ph) continue;
    const double lrr = m.flrr[f];
    const double2 mm = m.fm[f];
    const double c = lrr * (xv - xin[j]);
    tx = tx - c * (mm.x - xi.x);
    ty = ty - c * (mm.y - xi.y);
  }
  const double A = m.area[i];
  tmp[i] = make_double2(tx / A, ty / A);
}

// relaxation.jl:107-121
__global__ void k_mp_apply2(StateDev s, MeshDev m, int n, const double2* __restrict__ tmp, double* res) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = face_row(m, t);
  const int cap = m.cap, nf = m.nfaces[i];
  const double2 xi = s.x[i];
  const int ph = s.phase[i];
  const double2 ti = tmp[i];
  double r = 0.0;
  for (int k = 0; k < nf; ++k) {
    const size_t f = (size_t)k * cap + i;
    const int j = m.fnbr[f];
    if (s.phase[j] == ph) continue;
    const double lrr = m.flrr[f];
    const double2 mm = m.fm[f], y = m.fy[f];
    const double2 tj = tmp[j];
    const double zx = 0.5 * (xi.x + y.x), zy = 0.5 * (xi.y + y.y);
    const double a = (ti.x - tj.x) * (mm.x - zx) + (ti.y - tj.y) * (mm.y - zy);
    const double c = (ti.x + tj.x) * (xi.x - y.x) + (ti.y + tj.y) * (xi.y - y.y);
    r -= lrr * (a - 0.5 * c);
  }
  res[i] = r;
}

// relaxation.jl:190-204: dv += lrr (q_i - q_j)(m - x_i)/area on cross-phase faces
__global__ void k_mp_correct(StateDev s, MeshDev m, int n, const double* __restrict__ q, double threshold) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (s.quality[i] < threshold) return;
  const int cap = m.cap, nf = m.nfaces[i];
  const double2 xi = s.x[i];
  const int ph = s.phase[i];
  const double A = m.area[i];
  double2 d = s.dv[i];
  for (int k = 0; k < nf; ++k) {
    const size_t f = (size_t)k * cap + i;
    const int j = m.fnbr[f];
    if (s.phase[j] == ph) continue;
    const double lrr = m.flrr[f];
    const double2 mm = m.fm[f];
    const double c = lrr * (q[i] - q[j]);
    d.x = d.x + (c * (mm.x - xi.x)) / A;
    d.y = d.y + (c * (mm.y - xi.y)) / A;
  }
  s.dv[i] = d;
}

}  // namespace

// ------------------------------------------------------------------- host

#define LAUNCH_F(fam, kernel, ...)                                              \
  do {                                                                          \
    KernelTimer _kt(c, fam);                                                    \
    kernel<<<lv_blocks(c->n, TPB), TPB, 0, c->stream>>>(__VA_ARGS__);           \
    LV_LAUNCH_CHECK(c, #kernel);                                                \
  } while (0)
#define LAUNCH(kernel, ...) LAUNCH_F(LV_KF_OPS, kernel, __VA_ARGS__)

static int need_mesh(lv_ctx* c) {
  if (!c->meshed) return lv_fail(c, LV_ERR_NOT_MESHED, "the grid has not been meshed (call lv_remesh first)");
  return LV_OK;
}

int lv_phys_eos(lv_ctx* c, int kind, double gamma, double p) {
  if (int rc = need_mesh(c)) return rc;
  LAUNCH(k_eos, c->s, c->m, c->n, kind, gamma, p);
  return LV_OK;
}

int lv_phys_gravity(lv_ctx* c, double gx, double gy, double dt) {
  LAUNCH(k_gravity, c->s, c->n, gx, gy, dt);
  return LV_OK;
}

int lv_phys_pressure_step(lv_ctx* c, double dt) {
  if (int rc = need_mesh(c)) return rc;
  LAUNCH(k_pstep_v, c->s, c->m, c->n, dt);
  LAUNCH(k_pstep_e, c->s, c->m, c->n, dt);
  return LV_OK;
}

int lv_phys_rhs(lv_ctx* c, double dt, int gp_step, const double* vbc, int prepare, int guess, const float* D) {
  if (int rc = need_mesh(c)) return rc;
  if (prepare) {
    double w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (vbc)
      for (int k = 0; k < 8; ++k) w[k] = vbc[k];
    // vbc[4][2] indexed by -label-1: UP, RIGHT, DOWN, LEFT
    const Wall2 ud{w[0], w[1], w[4], w[5]};
    const Wall2 rl{w[2], w[3], w[6], w[7]};
    LAUNCH_F(LV_KF_RHS, k_rhs_prep, c->s, c->m, c->sv, c->n, dt, ud, rl, c->rhs_bvel,
             c->rhs_bvel ? c->bnd_off : nullptr);
  }
  static_assert(TPB == LV_SG_TPB, "the sweep-guess sums assume 256 threads per block");
  // the guess sums ride on the second pass (sweeps >= 2), on the first pass
  // of sweep 1 when there is a direction (the previous call's change)
  const int g1 = !guess ? 0 : (gp_step ? 1 : (D ? 2 : 0));
  LAUNCH_F(LV_KF_RHS, k_rhs, c->s, c->m, c->sv, c->n, dt, g1, D);
  if (gp_step) LAUNCH_F(LV_KF_RHS, k_rhs_gp, c->s, c->m, c->sv, c->n, guess, D);
  return LV_OK;
}

int lv_phys_find_D(lv_ctx* c) {
  if (int rc = need_mesh(c)) return rc;
  LAUNCH(k_find_D, c->s, c->m, c->n);
  return LV_OK;
}

int lv_phys_viscous(lv_ctx* c, double dt, int av) {
  if (int rc = need_mesh(c)) return rc;
  double2* Sa = reinterpret_cast<double2*>(c->sv.r);  // 2 x n doubles of scratch each
  double2* Sb = reinterpret_cast<double2*>(c->sv.p);
  const double avdr = av ? c->g.dr : 0.0;
  LAUNCH(k_stress, c->s, c->n, avdr, Sa, Sb);
  LAUNCH(k_visc_v, c->s, c->m, c->n, dt, Sa, Sb);
  LAUNCH(k_visc_e, c->s, c->m, c->n, dt, Sa, Sb);
  return LV_OK;
}

int lv_phys_friction(lv_ctx* c, const double* vwall, double dt, const double2* bvel, const unsigned char* act) {
  if (int rc = need_mesh(c)) return rc;
  double w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (vwall)
    for (int k = 0; k < 8; ++k) w[k] = vwall[k];
  const Wall2 ud{w[0], w[1], w[4], w[5]};
  const Wall2 rl{w[2], w[3], w[6], w[7]};
  LAUNCH(k_friction, c->s, c->m, c->n, dt, ud, rl, bvel, bvel ? c->bnd_off : nullptr, act);
  return LV_OK;
}

// ------------------------------------------------------ Fourier heat (fourier.jl)

// ideal_temperature! (fourier.jl:1-12): T = eint(p) / cV, eint = e - v.v / 2 (pressure.jl:32-34)
__global__ void k_ideal_temperature(StateDev s, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 v = s.v[i];
  s.T[i] = (s.e[i] - 0.5 * (v.x * v.x + v.y * v.y)) / s.cV[i];
}

// fourier_step! (fourier.jl:14-28): e -= dt k / m lrr (T_i - T_j), k = (k_i + k_j)/2, faces in order
__global__ void k_fourier(StateDev s, MeshDev m, int n, double dt) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = face_row(m, t);
  const int cap = m.cap, nf = m.nfaces[i];
  const double Ti = s.T[i], ki = s.kc[i], mi = s.mass[i];
  double e = s.e[i];
  for (int k0 = 0; k0 < nf; k0 += FB) {
    int j[FB];
    double lrr[FB], Tj[FB], kj[FB];
#pragma unroll
    for (int u = 0; u < FB; ++u) {
      const size_t f = face_slot(k0 + u, nf, cap, i);
      j[u] = ld_nc(m.fnbr + f);
      lrr[u] = ld_nc(m.flrr + f);
    }
#pragma unroll
    for (int u = 0; u < FB; ++u) {
      Tj[u] = ld_nc(s.T + j[u]);
      kj[u] = ld_nc(s.kc + j[u]);
    }
#pragma unroll
    for (int u = 0; u < FB; ++u) {
      if (k0 + u >= nf) break;
      const double k = 0.5 * (ki + kj[u]);
      e = e - dt * k / mi * lrr[u] * (Ti - Tj[u]);
    }
  }
  s.e[i] = e;
}

// heat_from_bdary! (fourier.jl:30-62): an implicit boundary heat flux from
// the wall temperatures Tb (per boundary edge, from boff[i] in edge order;
// NaN: adiabatic).  The reference asserts cV > 0: a boundary polygon without
// it raises LV_FLAG_BAD_INPUT and is left unchanged.
__global__ void k_heat_bdary(GridDev g, StateDev s, MeshDev m, int n, double dt, const double* __restrict__ Tb,
                             const int* __restrict__ boff, int* status) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = face_row(m, t);
  const int cap = m.cap, nf = m.nfaces[i], ne = m.nedges[i];
  if (nf == ne) return;  // !isboundary(p)
  const double cV = s.cV[i];
  if (!(cV > 0.0)) {
    atomicOr(status, LV_FLAG_BAD_INPUT);
    return;
  }
  const double2 xi = s.x[i], v = s.v[i];
  double implicit_factor = 1.0;
  const double thermal_D = s.kc[i] / (s.rho[i] * cV);
  const double e_kinetic = 0.5 * (v.x * v.x + v.y * v.y);
  double T = (s.e[i] - e_kinetic) / cV;
  const double A = m.area[i];
  int q = boff[i];
  for (int k = 0; k < ne; ++k) {
    const size_t f = (size_t)k * cap + i;
    if (m.elab[f] >= 0) continue;
    const double Tw = Tb[q++];
    const double2 a = m.ev1[f], b = m.ev2[f];
    const double mx = 0.5 * (a.x + b.x), my = 0.5 * (a.y + b.y);
    const double nx0 = a.y - b.y, ny0 = b.x - a.x;
    const double nn = sqrt(nx0 * nx0 + ny0 * ny0);
    const double nx = nx0 / nn, ny = ny0 / nn;
    const double lx = a.x - b.x, ly = a.y - b.y;
    const double len = sqrt(lx * lx + ly * ly);
    const double lrr = len / fabs((mx - xi.x) * nx + (my - xi.y) * ny) + 0.01 * g.dr;
    if (!isnan(Tw)) {
      const double tmp = dt * thermal_D * lrr / A;
      T = T + tmp * Tw;
      implicit_factor = implicit_factor + tmp;
    }
  }
  T = T / implicit_factor;
  s.T[i] = T;
  s.e[i] = e_kinetic + cV * T;
}

// ------------------------------------------------------ implicit viscosity (viscous_solver.jl)

// ViscousSolver assemble! (viscous_solver.jl:79-107): per particle the
// neighbours' entries -0.5 lrr (mu_i + mu_j) in face order and the self entry
// vv = m/dt minus them (the rows of both velocity components hold the same
// entries); b = (m/dt) v and the first guess v, interleaved (v_index).
__global__ void k_visc_sys(StateDev s, MeshDev m, int n, double dt, const int* __restrict__ rowptr, int* col,
                           double* w, double* diag, double* b, double* u0) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = face_row(m, t);
  const int cap = m.cap, nf = m.nfaces[i];
  const double mi = s.mass[i], mui = s.mu[i];
  const double2 v = s.v[i];
  const int base = rowptr[i];
  b[2 * (size_t)i] = mi / dt * v.x;
  b[2 * (size_t)i + 1] = mi / dt * v.y;
  u0[2 * (size_t)i] = v.x;
  u0[2 * (size_t)i + 1] = v.y;
  double vv = mi / dt;
  for (int k = 0; k < nf; ++k) {
    const size_t f = (size_t)k * cap + i;
    const int j = m.fnbr[f];
    const double wv = -0.5 * m.flrr[f] * (mui + s.mu[j]);
    col[base + k] = j;
    w[base + k] = wv;
    vv = vv - wv;
  }
  diag[i] = vv;
}

__global__ void k_visc_store(StateDev s, int n, const double* __restrict__ u) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) s.v[i] = make_double2(u[2 * (size_t)i], u[2 * (size_t)i + 1]);
}

int lv_phys_ideal_temperature(lv_ctx* c) {
  LAUNCH(k_ideal_temperature, c->s, c->n);
  return LV_OK;
}

int lv_phys_fourier(lv_ctx* c, double dt) {
  if (int rc = need_mesh(c)) return rc;
  LAUNCH(k_fourier, c->s, c->m, c->n, dt);
  return LV_OK;
}

int lv_phys_heat_bdary(lv_ctx* c, int64_t nb, const double* Tb, double dt) {
  if (int rc = lv_bnd_prepare(c)) return rc;
  if (nb != c->bnd_count || (nb > 0 && !Tb))
    return lv_fail(c, LV_ERR_BAD_ARGUMENT, "heat_from_bdary!: nb is not the mesh's boundary-edge count");
  double* dTb = reinterpret_cast<double*>(c->bnd_vel);  // room for 2 nb doubles
  if (nb > 0) cudaMemcpyAsync(dTb, Tb, sizeof(double) * (size_t)nb, cudaMemcpyHostToDevice, c->stream);
  LAUNCH(k_heat_bdary, c->g, c->s, c->m, c->n, dt, dTb, c->bnd_off, c->status);
  return LV_OK;
}

// viscous_step!(solver::ViscousSolver, dt) (viscous_solver.jl:109-129): the
// implicit system solved by MINRES with atol = rtol = 1e-6, itmax = 2000
// (the device MINRES on the 2n interleaved unknowns, the ThreadedMat row
// form), then v = the solution.  Statistics into stats slot 31.
int lv_phys_viscous_implicit(lv_ctx* c, double dt) {
  if (int rc = need_mesh(c)) return rc;
  const int n = c->n;
  if (!c->vs_col) {
    bool ok = cudaMalloc(&c->vs_rowptr, sizeof(int) * ((size_t)c->cap + 1)) == cudaSuccess;
    ok = ok && cudaMalloc(&c->vs_col, sizeof(int) * (size_t)c->sv.nnz_cap) == cudaSuccess;
    ok = ok && cudaMalloc(&c->vs_w, sizeof(double) * (size_t)c->sv.nnz_cap) == cudaSuccess;
    ok = ok && cudaMalloc(&c->vs_diag, sizeof(double) * (size_t)c->cap) == cudaSuccess;
    ok = ok && cudaMalloc(&c->vs_b, sizeof(double) * 2 * (size_t)c->cap) == cudaSuccess;
    ok = ok && cudaMalloc(&c->vs_u, sizeof(double) * 2 * (size_t)c->cap) == cudaSuccess;
    for (void* p : {(void*)c->vs_rowptr, (void*)c->vs_col, (void*)c->vs_w, (void*)c->vs_diag, (void*)c->vs_b,
                    (void*)c->vs_u})
      if (p) c->allocs.push_back(p);
    if (!ok) {
      c->vs_col = nullptr;
      return lv_fail(c, LV_ERR_CUDA, "allocation of the viscous system failed");
    }
  }
  {
    KernelTimer kt(c, LV_KF_OPS);
    if (int rc = lv_scan_int(c, c->m.nfaces, c->vs_rowptr, n)) return rc;
    k_visc_sys<<<lv_blocks(n, TPB), TPB, 0, c->stream>>>(c->s, c->m, n, dt, c->vs_rowptr, c->vs_col, c->vs_w,
                                                          c->vs_diag, c->vs_b, c->vs_u);
    LV_LAUNCH_CHECK(c, "k_visc_sys");
  }
  {
    KernelTimer kt(c, LV_KF_PCG);
    if (int rc = lv_minres_general(c, c->vs_rowptr, c->vs_col, c->vs_w, c->vs_diag, c->vs_b, c->vs_u, 2, 1, 1e-6,
                                   2000, LV_VISC_SLOT))
      return rc;
  }
  LAUNCH(k_visc_store, c->s, n, c->vs_u);
  return LV_OK;
}

// ------------------------------------------------------ boundary edges
//
// The boundary edges of the current mesh in the order of boundaries(p)
// (iterators.jl:46-57) over the polygons: polygon i's edges start at
// bnd_off[i] (a scan of the per-polygon counts, built once per mesh).

__global__ void k_bnd_count(MeshDev m, int n, int* cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) cnt[i] = m.nedges[i] - m.nfaces[i];
}

__global__ void k_bnd_list(MeshDev m, int n, const int* __restrict__ off, double2* mid, int* lab) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int cap = m.cap, ne = m.nedges[i];
  int q = off[i];
  for (int k = 0; k < ne; ++k) {
    const size_t f = (size_t)k * cap + i;
    const int l = m.elab[f];
    if (l >= 0) continue;
    const double2 a = m.ev1[f], b = m.ev2[f];
    mid[q] = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y + b.y));  // midpoint(e), geometry.jl:145-147
    lab[q] = l;
    ++q;
  }
}

// Offsets and count of the current mesh's boundary edges (synchronises once
// per mesh) and room for per-edge values.
int lv_bnd_prepare(lv_ctx* c) {
  if (int rc = need_mesh(c)) return rc;
  if (c->bnd_valid) return LV_OK;
  const int n = c->n;
  if (!c->bnd_off) {
    if (cudaMalloc(&c->bnd_off, sizeof(int) * ((size_t)c->cap + 1)) != cudaSuccess ||
        cudaMalloc(&c->bnd_cnt, sizeof(int) * (size_t)c->cap) != cudaSuccess)
      return lv_fail(c, LV_ERR_CUDA, "allocation of the boundary-edge offsets failed");
    c->allocs.push_back(c->bnd_off);
    c->allocs.push_back(c->bnd_cnt);
  }
  k_bnd_count<<<lv_blocks(n, TPB), TPB, 0, c->stream>>>(c->m, n, c->bnd_cnt);
  LV_LAUNCH_CHECK(c, "k_bnd_count");
  if (int rc = lv_scan_int(c, c->bnd_cnt, c->bnd_off, n)) return rc;
  int total = 0;
  cudaMemcpyAsync(&total, c->bnd_off + n, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (int rc = lv_cuda_check(c, cudaStreamSynchronize(c->stream), "boundary edges")) return rc;
  if (total > c->bnd_room) {
    cudaFree(c->bnd_vel);
    cudaFree(c->bnd_act);
    cudaFree(c->bnd_lab);
    c->bnd_vel = nullptr;
    c->bnd_act = nullptr;
    c->bnd_lab = nullptr;
    c->bnd_room = 0;
    const size_t room = (size_t)total + 1024;
    if (cudaMalloc(&c->bnd_vel, sizeof(double2) * room) != cudaSuccess ||
        cudaMalloc(&c->bnd_act, room) != cudaSuccess || cudaMalloc(&c->bnd_lab, sizeof(int) * room) != cudaSuccess)
      return lv_fail(c, LV_ERR_CUDA, "allocation of the boundary-edge values failed");
    c->bnd_room = (int)room;
  }
  c->bnd_count = total;
  c->bnd_valid = true;
  return LV_OK;
}

int lv_bnd_list(lv_ctx* c, double* mid, int* lab) {
  if (int rc = lv_bnd_prepare(c)) return rc;
  const int nb = c->bnd_count;
  if (nb == 0) return LV_OK;
  k_bnd_list<<<lv_blocks(c->n, TPB), TPB, 0, c->stream>>>(c->m, c->n, c->bnd_off, c->bnd_vel, c->bnd_lab);
  LV_LAUNCH_CHECK(c, "k_bnd_list");
  if (mid) cudaMemcpyAsync(mid, c->bnd_vel, sizeof(double2) * nb, cudaMemcpyDeviceToHost, c->stream);
  if (lab) cudaMemcpyAsync(lab, c->bnd_lab, sizeof(int) * nb, cudaMemcpyDeviceToHost, c->stream);
  return lv_cuda_check(c, cudaStreamSynchronize(c->stream), "boundary edges");
}

// Uploads per-edge values (nb must be the current count); act may be null.
int lv_bnd_upload(lv_ctx* c, int64_t nb, const double* vb, const unsigned char* act) {
  if (int rc = lv_bnd_prepare(c)) return rc;
  if (nb != c->bnd_count || (nb > 0 && !vb))
    return lv_fail(c, LV_ERR_BAD_ARGUMENT, "per-edge boundary values: nb is not the mesh's boundary-edge count");
  if (nb == 0) return LV_OK;
  cudaMemcpyAsync(c->bnd_vel, vb, sizeof(double2) * (size_t)nb, cudaMemcpyHostToDevice, c->stream);
  if (act) cudaMemcpyAsync(c->bnd_act, act, (size_t)nb, cudaMemcpyHostToDevice, c->stream);
  return lv_cuda_check(c, cudaGetLastError(), "boundary values upload");
}

int lv_phys_find_dv(lv_ctx* c, double dt, double alpha) {
  if (int rc = need_mesh(c)) return rc;
  LAUNCH(k_find_dv, c->s, c->m, c->n, dt, alpha);
  return LV_OK;
}

int lv_phys_relax(lv_ctx* c, double dt, int rusanov) {
  if (int rc = need_mesh(c)) return rc;
  double* ndv = c->sv.q;  // scratch between solves
  if (rusanov) {
    LAUNCH(k_norm_dv, c->s, c->m, c->n, ndv, c->flen_valid ? 0 : 1);
    c->flen_valid = true;
  }
  LAUNCH(k_relax_flux, c->s, c->m, c->n, dt, rusanov, ndv);
  LAUNCH(k_relax_update, c->s, c->n, dt);
  c->meshed = false;
  return lv_mesh_remesh(c);
}

int lv_phys_move(lv_ctx* c, double dt) {
  if (int rc = need_mesh(c)) return rc;
  LAUNCH(k_move, c->g, c->s, c->m, c->n, dt, c->status);
  c->meshed = false;
  return lv_mesh_remesh(c);
}

// MINRES (Paige & Saunders 1975) on the multiphase projector, with the
// vectors on the device and the scalar recurrences on the host; it is used
// only by the two-phase workload and runs at most itmax = 200 iterations
// (relaxation.jl:182).
int lv_phys_multiphase(lv_ctx* c, double threshold, lv_solve_stats* st);

namespace {

// two dot products, block partials (fixed order within a block)
__global__ void k_dot2(int n, const double* __restrict__ a, const double* __restrict__ b,
                       const double* __restrict__ c, const double* __restrict__ d, double* part) {
  __shared__ double sh[2][32];
  double s0 = 0.0, s1 = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    s0 += a[i] * b[i];
    if (c) s1 += c[i] * d[i];
  }
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_down_sync(0xffffffffu, s0, o);
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    sh[0][wid] = s0;
    sh[1][wid] = s1;
  }
  __syncthreads();
  if (wid == 0) {
    s0 = lane < (int)(blockDim.x >> 5) ? sh[0][lane] : 0.0;
    s1 = lane < (int)(blockDim.x >> 5) ? sh[1][lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      s0 += __shfl_down_sync(0xffffffffu, s0, o);
      s1 += __shfl_down_sync(0xffffffffu, s1, o);
    }
    if (lane == 0) {
      part[2 * blockIdx.x] = s0;
      part[2 * blockIdx.x + 1] = s1;
    }
  }
}

__global__ void k_dot2_final(int nb, const double* part, double* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s0 = 0.0, s1 = 0.0;
  for (int b = 0; b < nb; ++b) {
    s0 += part[2 * b];
    s1 += part[2 * b + 1];
  }
  out[0] = s0;
  out[1] = s1;
}

// y = alpha x + beta y (element-wise)
__global__ void k_axpby(int n, double alpha, const double* __restrict__ x, double beta, double* y) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = alpha * x[i] + beta * y[i];
}

// MINRES direction update: w = (v - oldeps w1 - delta w2) denom; q += phi w
__global__ void k_minres_update(int n, const double* __restrict__ v, const double* __restrict__ w1,
                                const double* __restrict__ w2, double* w, double* q, double oldeps, double delta,
                                double denom, double phi) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double wi = (v[i] - oldeps * w1[i] - delta * w2[i]) * denom;
  w[i] = wi;
  q[i] += phi * wi;
}

}  // namespace

// multiphase_projection! (relaxation.jl:180-206): refresh! of b, MINRES on
// the projector (atol = rtol = 1e-4, itmax = 200, zero initial guess; Paige &
// Saunders 1975 with the stopping rule ||r|| <= atol + rtol ||r0||), then the
// dv correction on cross-phase faces of polygons with quality >= threshold.
int lv_phys_multiphase(lv_ctx* c, double threshold, lv_solve_stats* st) {
  if (int rc = need_mesh(c)) return rc;
  const int n = c->n;
  cudaStream_t s = c->stream;
  static thread_local double* host2 = nullptr;
  if (!host2 && cudaMallocHost(&host2, 2 * sizeof(double)) != cudaSuccess)
    return lv_fail(c, LV_ERR_CUDA, "pinned buffer");
  // device vectors: b, q, r1, r2, y, v, w, w1, w2, tmp2 (2n), part
  const size_t cap = c->cap;
  if (!c->mp_buf) {
    // 11 vectors + block partials (2 x 4096) + the two final sums
    if (cudaMalloc(&c->mp_buf, sizeof(double) * (11 * cap + 2 * 4096 + 64)) != cudaSuccess)
      return lv_fail(c, LV_ERR_CUDA, "multiphase buffers");
    c->allocs.push_back(c->mp_buf);
  }
  double* B = c->mp_buf;
  double *b = B, *q = B + cap, *r1 = B + 2 * cap, *r2 = B + 3 * cap, *y = B + 4 * cap, *v = B + 5 * cap,
         *w = B + 6 * cap, *w1 = B + 7 * cap, *w2 = B + 8 * cap;
  double2* tmp = reinterpret_cast<double2*>(B + 9 * cap);
  double* part = B + 11 * cap;
  const int nb = std::min(4096, lv_blocks(n, TPB));
  auto dots = [&](const double* a1, const double* b1, const double* a2, const double* b2, double& o0,
                  double& o1) -> int {
    k_dot2<<<nb, TPB, 0, s>>>(n, a1, b1, a2, b2, part);
    k_dot2_final<<<1, 32, 0, s>>>(nb, part, part + 2 * 4096);
    c->launches += 2;
    cudaMemcpyAsync(host2, part + 2 * 4096, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return lv_cuda_check(c, e, "multiphase dot");
    o0 = host2[0];
    o1 = host2[1];
    return LV_OK;
  };
  auto apply = [&](const double* xin, double* res) -> int {
    LAUNCH(k_mp_apply1, c->s, c->m, n, xin, tmp);
    LAUNCH(k_mp_apply2, c->s, c->m, n, tmp, res);
    return LV_OK;
  };
  LAUNCH(k_mp_rhs, c->s, c->m, n, b);
  cudaMemsetAsync(q, 0, sizeof(double) * n, s);
  cudaMemsetAsync(w, 0, sizeof(double) * n, s);
  cudaMemsetAsync(w2, 0, sizeof(double) * n, s);
  cudaMemcpyAsync(r1, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(y, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
  double beta1 = 0.0, dummy = 0.0;
  if (int rc = dots(r1, y, nullptr, nullptr, beta1, dummy)) return rc;
  beta1 = sqrt(beta1);
  const double tol = 1e-4;
  const int itmax = 200;
  int itn = 0;
  bool solved = beta1 == 0.0;
  if (!solved) {
    cudaMemcpyAsync(r2, r1, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
    double oldb = 0.0, beta = beta1, dbar = 0.0, epsln = 0.0, phibar = beta1, cs = -1.0, sn = 0.0, tnorm2 = 0.0;
    const double eps = 2.220446049250313e-16;
    const double tl = tol + tol * beta1;
    while (itn < itmax) {
      ++itn;
      LAUNCH(k_axpby, n, 1.0 / beta, y, 0.0, v);
      if (int rc = apply(v, y)) return rc;
      if (itn >= 2) LAUNCH(k_axpby, n, -(beta / oldb), r1, 1.0, y);
      double alfa = 0.0;
      if (int rc = dots(v, y, nullptr, nullptr, alfa, dummy)) return rc;
      LAUNCH(k_axpby, n, -(alfa / beta), r2, 1.0, y);
      std::swap(r1, r2);
      cudaMemcpyAsync(r2, y, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
      oldb = beta;
      double bb = 0.0;
      if (int rc = dots(r2, y, nullptr, nullptr, bb, dummy)) return rc;
      beta = sqrt(bb > 0.0 ? bb : 0.0);
      tnorm2 += alfa * alfa + oldb * oldb + beta * beta;
      const double oldeps = epsln, delta = cs * dbar + sn * alfa, gbar = sn * dbar - cs * alfa;
      epsln = sn * beta;
      dbar = -cs * beta;
      const double root = sqrt(gbar * gbar + dbar * dbar);
      const double gamma = std::max(sqrt(gbar * gbar + beta * beta), eps);
      cs = gbar / gamma;
      sn = beta / gamma;
      const double phi = cs * phibar;
      phibar = sn * phibar;
      const double denom = 1.0 / gamma;
      std::swap(w1, w2);
      std::swap(w2, w);
      LAUNCH(k_minres_update, n, v, w1, w2, w, q, oldeps, delta, denom, phi);
      const double Anorm = sqrt(tnorm2), Arnorm = phibar * root;
      if (phibar <= tl || beta == 0.0 || (Anorm > 0 && phibar > 0 && Arnorm / (Anorm * phibar) <= tol)) {
        solved = true;
        break;
      }
    }
  }
  LAUNCH(k_mp_correct, c->s, c->m, n, q, threshold);
  if (st) {
    st->iterations = itn;
    st->converged = solved ? 1 : 0;
    st->outer = 0;
    st->method = -1;
    st->rel_residual = 0.0;
  }
  return LV_OK;
}
