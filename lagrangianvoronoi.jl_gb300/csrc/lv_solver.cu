// Pressure operator assembly and the pressure solve.
//
// PressureOperator refresh! (src/pressure.jl:104-117) is assembled into a
// device CSR: rowptr from a scan of the per-polygon face counts, col = the
// neighbour index, w = lr_ratio * (0.5/rho_i + 0.5/rho_j) in the face order
// of `neighbors`.  The reference applies the operator as
//     y_i = diag_i x_i + sum_j w_ij (x_i - x_j)          (pressure.jl:119-130)
// which the solver evaluates in the equivalent CSR form
//     y_i = adiag_i x_i - sum_j w_ij x_j,   adiag_i = diag_i + sum_j w_ij,
// one fused multiply-add per nonzero.
//
// The FP64 Jacobi-PCG runs as ONE persistent cooperative kernel per linear
// solve: the blocks meet at bounded grid barriers (two per iteration), each
// block reduces its rows' partial dot products, and every block sums the
// partials in the same fixed order, so all blocks take the same convergence
// decision and the result does not depend on scheduling.  The search
// direction update is folded into the matrix-vector product
// (q = A z + beta q, p = z + beta p), which leaves two barriers per
// iteration instead of three.
#include <math.h>

#include <algorithm>
#include <mutex>

#include "lv_internal.cuh"

namespace {

constexpr int TPB = 256;
constexpr int CG_TPB = 256;

// (also clears the nonsingular flag that k_assemble then sets)
__global__ void k_half_rho(const double* __restrict__ rho, double* hr, int n, int* nonsingular) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) *nonsingular = 0;
  if (i < n) hr[i] = 0.5 / rho[i];
}

// refresh!(A, grid, dt) (pressure.jl:104-117) into CSR.
// Also the FP32 copies of w, diag and dinv (the mixed solvers and the sweep
// guess) and the flag of a nonsingular operator (some diagonal term != 0).
__global__ void k_assemble(StateDev s, MeshDev m, SolverDev sv, int n, double dt, const double* __restrict__ hr,
                           int* nonsingular) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = face_row(m, t);
  const int cap = m.cap, nf = m.nfaces[i];
  const double rho = s.rho[i];
  const double diag = s.mass[i] / (rho * rho * s.c2[i] * (dt * dt));
  const double hi = hr[i];
  const int base = sv.rowptr[i];
  double ad = diag;
  for (int k = 0; k < nf; ++k) {
    const size_t f = (size_t)k * cap + i;
    const int j = m.fnbr[f];
    const double w = m.flrr[f] * (hi + hr[j]);
    sv.col[base + k] = j;
    sv.w[base + k] = w;
    sv.w32[base + k] = (float)w;
    if (sv.ew64) {  // the streaming solver's slot-major copies
      sv.ew64[f] = w;
      sv.ew32[f] = (float)w;
    }
    ad += w;
  }
  const double dinv = 1.0 / ad;
  sv.diag[i] = diag;
  sv.adiag[i] = ad;
  sv.dinv[i] = dinv;
  sv.d32[i] = (float)diag;
  sv.dinv32[i] = (float)dinv;
  if (diag != 0.0) atomicOr(nonsingular, 1);
}

__global__ void k_spmv(int n, const int* __restrict__ rowptr, const int* __restrict__ col, const double* __restrict__ w,
                       const double* __restrict__ adiag, const double* __restrict__ x, double* y) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double acc = adiag[i] * x[i];
  for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) acc -= w[k] * x[col[k]];
  y[i] = acc;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid barrier for a cooperative launch (all blocks co-resident).
// bar[0] is an arrival word, zeroed by the host before the launch: block 0
// adds 2^31 - (nblocks - 1), every other block adds 1, so the word's top bit
// flips exactly when the last block arrives and its low bits return to zero
// for the next barrier.  Every wait is bounded: after `limit` clock cycles
// (about 2 s by default) the block records LV_FLAG_BARRIER_TIMEOUT and the
// caller leaves the kernel.
__device__ bool grid_barrier(unsigned* bar, int* status, long long limit) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned inc = (blockIdx.x == 0) ? (0x80000000u - (gridDim.x - 1)) : 1u;
    __threadfence();
    const unsigned old = atomicAdd(bar, inc);
    const long long t0 = clock64();
    while (((old ^ ld_acquire_u32(bar)) & 0x80000000u) == 0u) {
      if (clock64() - t0 > limit) {
        atomicOr(status, LV_FLAG_BARRIER_TIMEOUT);
        ok = 0;
        break;
      }
    }
    __threadfence();
    if (ok && (ld_acquire_u32(reinterpret_cast<unsigned*>(status)) & LV_FLAG_BARRIER_TIMEOUT)) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Sum over the block (fixed order); result valid in thread 0.
template <int NV>
__device__ void block_sums(double (&v)[NV], double* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double t = warp_sum(v[k]);
    if (lane == 0) sh[k * 32 + wid] = t;
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double t = (lane < (int)(blockDim.x >> 5)) ? sh[k * 32 + lane] : 0.0;
      v[k] = warp_sum(t);
    }
  }
  __syncthreads();
}

// Sum of the per-block partials of `slot` in a fixed order, broadcast to all
// threads of the block.
__device__ double grid_total(const double* part, int slot, double* sh) {
  __shared__ double s_tot;
  if (threadIdx.x < 32) {
    double t = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += 32) t += part[slot * gridDim.x + b];
    t = warp_sum(t);
    if (threadIdx.x == 0) s_tot = t;
  }
  __syncthreads();
  double r = s_tot;
  __syncthreads();
  return r;
}

struct PCGArgs {
  int n;
  const int* rowptr;
  const int* col;
  const double* w;
  const double* adiag;
  const double* dinv;
  const double* b;
  double* x;
  double *r, *z, *p, *q;
  double* part;
  unsigned* bar;
  int* status;
  double tol2;
  int itmax;
  long long spin;          // cycles a grid barrier waits before it gives up
  const int* nonsingular;  // set by k_assemble when some diagonal term is nonzero
  const double* diag;      // the reference's diagonal term (mixed solver only)
  int* out_iters;
  double* out_d;  // [rr, bb, true rr]
  long long* counters;
};

// Jacobi-preconditioned CG, stopping when ||r||^2 <= tol^2 ||b||^2 (recursive
// residual) or after itmax iterations.  For a singular operator (no diagonal
// term anywhere) b is replaced by b - mean(b).
__global__ void __launch_bounds__(CG_TPB) k_pcg(PCGArgs a) {
  __shared__ double sh[4 * 32];
  const int n = a.n;
  const int stride = gridDim.x * blockDim.x;
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
  const int nb = gridDim.x;
  double bmean = 0.0;
  if (*a.nonsingular == 0) {
    double v[1] = {0.0};
    for (int i = t0; i < n; i += stride) v[0] += a.b[i];
    block_sums<1>(v, sh);
    if (threadIdx.x == 0) a.part[3 * nb + blockIdx.x] = v[0];
    if (!grid_barrier(a.bar, a.status, a.spin)) return;
    bmean = grid_total(a.part, 3, sh) / (double)n;
    if (!grid_barrier(a.bar, a.status, a.spin)) return;
  }
  // r = b - A x, z = M^-1 r, p = q = 0
  {
    double v[3] = {0.0, 0.0, 0.0};
    for (int i = t0; i < n; i += stride) {
      double acc = a.adiag[i] * a.x[i];
      for (int k = a.rowptr[i]; k < a.rowptr[i + 1]; ++k) acc -= a.w[k] * __ldcg(a.x + a.col[k]);
      const double bi = a.b[i] - bmean;
      const double ri = bi - acc;
      const double zi = a.dinv[i] * ri;
      a.r[i] = ri;
      a.z[i] = zi;
      a.p[i] = 0.0;
      a.q[i] = 0.0;
      v[0] += ri * zi;
      v[1] += ri * ri;
      v[2] += bi * bi;
    }
    block_sums<3>(v, sh);
    if (threadIdx.x == 0) {
      a.part[1 * nb + blockIdx.x] = v[0];
      a.part[2 * nb + blockIdx.x] = v[1];
      a.part[3 * nb + blockIdx.x] = v[2];
    }
  }
  if (!grid_barrier(a.bar, a.status, a.spin)) return;
  double rz = grid_total(a.part, 1, sh);
  double rr = grid_total(a.part, 2, sh);
  const double bb = grid_total(a.part, 3, sh);
  double beta = 0.0;
  int it = 0;
  while (!(rr <= a.tol2 * bb) && it < a.itmax) {
    // p = z + beta p;  q = A z + beta q  (= A p)
    {
      double v[1] = {0.0};
      for (int i = t0; i < n; i += stride) {
        const double zi = a.z[i];
        double acc = a.adiag[i] * zi;
        for (int k = a.rowptr[i]; k < a.rowptr[i + 1]; ++k) acc -= a.w[k] * __ldcg(a.z + a.col[k]);
        const double pi = zi + beta * a.p[i];
        const double qi = acc + beta * a.q[i];
        a.p[i] = pi;
        a.q[i] = qi;
        v[0] += pi * qi;
      }
      block_sums<1>(v, sh);
      if (threadIdx.x == 0) a.part[0 * nb + blockIdx.x] = v[0];
    }
    if (!grid_barrier(a.bar, a.status, a.spin)) return;
    const double alpha = rz / grid_total(a.part, 0, sh);
    {
      double v[2] = {0.0, 0.0};
      for (int i = t0; i < n; i += stride) {
        a.x[i] += alpha * a.p[i];
        const double ri = a.r[i] - alpha * a.q[i];
        const double zi = a.dinv[i] * ri;
        a.r[i] = ri;
        a.z[i] = zi;
        v[0] += ri * zi;
        v[1] += ri * ri;
      }
      block_sums<2>(v, sh);
      if (threadIdx.x == 0) {
        a.part[1 * nb + blockIdx.x] = v[0];
        a.part[2 * nb + blockIdx.x] = v[1];
      }
    }
    if (!grid_barrier(a.bar, a.status, a.spin)) return;
    const double rz_new = grid_total(a.part, 1, sh);
    rr = grid_total(a.part, 2, sh);
    beta = rz_new / rz;
    rz = rz_new;
    ++it;
  }
  // true residual of the final iterate
  {
    double v[1] = {0.0};
    for (int i = t0; i < n; i += stride) {
      double acc = a.adiag[i] * a.x[i];
      for (int k = a.rowptr[i]; k < a.rowptr[i + 1]; ++k) acc -= a.w[k] * __ldcg(a.x + a.col[k]);
      const double ri = (a.b[i] - bmean) - acc;
      v[0] += ri * ri;
    }
    block_sums<1>(v, sh);
    if (threadIdx.x == 0) a.part[0 * nb + blockIdx.x] = v[0];
  }
  if (!grid_barrier(a.bar, a.status, a.spin)) return;
  if (blockIdx.x == 0) {
    const double tr = grid_total(a.part, 0, sh);
    if (threadIdx.x == 0) {
      *a.out_iters = it;
      count_solve(a.counters, it, rr, bb, tr, a.tol2);
      a.out_d[0] = rr;
      a.out_d[1] = bb;
      a.out_d[2] = tr;
    }
  }
}

// ---------------------------------------------------------------------------
// Register-resident pipelined Jacobi-PCG for systems whose rows fit in the
// registers of one cooperative grid (at most R rows per thread).
//
// Pipelined CG (Ghysels & Vanroose, Parallel Computing 40, 2014, Alg. 3)
// needs one global reduction and one matrix-vector product per iteration,
// and the product can start before the reduction finishes, so each iteration
// costs a single grid barrier.  Every thread keeps its rows' CSR entries (the
// first KR of each row) and all eight CG vectors in registers; the only
// vectors exchanged through global memory are m = M^-1 w (double-buffered by
// iteration parity) and, at (re)starts, u and x.  The recursive residual is
// confirmed by an explicit residual b - A x before the kernel exits; if it
// misses the tolerance, CG restarts from it (at most 3 times).
// ---------------------------------------------------------------------------
constexpr int SP_TPB = 128;
constexpr int KR = 8;

template <int R>
struct RowRegs {
  int i[R];
  int beg[R], cnt[R];
  int cc[R][KR];
  double ww[R][KR];
  double adg[R], dnv[R], bb[R];
};

// Values other blocks wrote during this kernel are read with __ldcg (L2, not
// the non-coherent L1 / read-only paths).
template <int R>
__device__ __forceinline__ void row_apply(const RowRegs<R>& rr, const PCGArgs& a, const double* __restrict__ vg,
                                          const double (&own)[R], double (&out)[R]) {
#pragma unroll
  for (int r = 0; r < R; ++r) {
    double acc = rr.adg[r] * own[r];
#pragma unroll
    for (int k = 0; k < KR; ++k)
      if (k < rr.cnt[r]) acc -= rr.ww[r][k] * __ldcg(vg + rr.cc[r][k]);
    for (int k = KR; k < rr.cnt[r]; ++k) acc -= a.w[rr.beg[r] + k] * __ldcg(vg + a.col[rr.beg[r] + k]);
    out[r] = acc;
  }
}

template <int NV>
__device__ void grid_totals(const double* part, int slot0, double (&tot)[NV]) {
  __shared__ double s_tot[NV];
  if (threadIdx.x < 32) {
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double t = 0.0;
      for (int b = threadIdx.x; b < (int)gridDim.x; b += 32) t += part[(slot0 + v) * gridDim.x + b];
      t = warp_sum(t);
      if (threadIdx.x == 0) s_tot[v] = t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int v = 0; v < NV; ++v) tot[v] = s_tot[v];
  __syncthreads();
}

template <int R>
__global__ void __launch_bounds__(SP_TPB) k_pcg_reg(PCGArgs a, double* ubuf, double* mbuf0, double* mbuf1) {
  __shared__ double sh[4 * 32];
  const int n = a.n;
  const int nb = gridDim.x;
  const int stride = gridDim.x * blockDim.x;
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
  RowRegs<R> rr;
  double x[R], r[R], u[R], w[R], z[R], q[R], s[R], p[R], m[R];
#pragma unroll
  for (int k = 0; k < R; ++k) {
    const int i = t0 + k * stride;
    rr.i[k] = i;
    const bool on = i < n;
    rr.beg[k] = on ? a.rowptr[i] : 0;
    rr.cnt[k] = on ? a.rowptr[i + 1] - rr.beg[k] : 0;
#pragma unroll
    for (int e = 0; e < KR; ++e) {
      const bool have = e < rr.cnt[k];
      rr.cc[k][e] = have ? a.col[rr.beg[k] + e] : 0;
      rr.ww[k][e] = have ? a.w[rr.beg[k] + e] : 0.0;
    }
    rr.adg[k] = on ? a.adiag[i] : 0.0;
    rr.dnv[k] = on ? a.dinv[i] : 0.0;
    rr.bb[k] = on ? a.b[i] : 0.0;
    x[k] = on ? a.x[i] : 0.0;
  }
  // singular operator: project b to zero mean
  if (*a.nonsingular == 0) {
    double v[1] = {0.0};
#pragma unroll
    for (int k = 0; k < R; ++k) v[0] += rr.bb[k];
    block_sums<1>(v, sh);
    if (threadIdx.x == 0) a.part[0 * nb + blockIdx.x] = v[0];
    if (!grid_barrier(a.bar, a.status, a.spin)) return;
    double t[1];
    grid_totals<1>(a.part, 0, t);
    const double mean = t[0] / (double)n;
#pragma unroll
    for (int k = 0; k < R; ++k)
      if (rr.i[k] < n) rr.bb[k] -= mean;
    if (!grid_barrier(a.bar, a.status, a.spin)) return;
  }
  int it = 0;
  double bnorm2 = 0.0, rtrue2 = 0.0, rho = 0.0;
  for (int attempt = 0; attempt < 4; ++attempt) {
    // r = b - A x (x exchanged through a.x), u = M^-1 r
    double ax[R];
    row_apply<R>(rr, a, a.x, x, ax);
    double v[2] = {0.0, 0.0};
#pragma unroll
    for (int k = 0; k < R; ++k) {
      const bool on = rr.i[k] < n;
      r[k] = on ? rr.bb[k] - ax[k] : 0.0;
      u[k] = rr.dnv[k] * r[k];
      if (on) ubuf[rr.i[k]] = u[k];
      v[0] += r[k] * r[k];
      v[1] += rr.bb[k] * rr.bb[k];
    }
    block_sums<2>(v, sh);
    if (threadIdx.x == 0) {
      a.part[0 * nb + blockIdx.x] = v[0];
      a.part[1 * nb + blockIdx.x] = v[1];
    }
    if (!grid_barrier(a.bar, a.status, a.spin)) return;
    double t2[2];
    grid_totals<2>(a.part, 0, t2);
    rtrue2 = t2[0];
    bnorm2 = t2[1];
    if (rtrue2 <= a.tol2 * bnorm2 || it >= a.itmax) break;
    // w = A u
    row_apply<R>(rr, a, ubuf, u, w);
    double gamma_old = 1.0, alpha_old = 1.0;  // meaningful in thread 0 only
    bool first = true;
    const int it_first = it;
    int parity = 0;
    while (true) {
      double* mb = parity ? mbuf1 : mbuf0;
      double v3[3] = {0.0, 0.0, 0.0};
#pragma unroll
      for (int k = 0; k < R; ++k) {
        v3[0] += r[k] * u[k];
        v3[1] += w[k] * u[k];
        v3[2] += r[k] * r[k];
        m[k] = rr.dnv[k] * w[k];
        if (rr.i[k] < n) mb[rr.i[k]] = m[k];
      }
      block_sums<3>(v3, sh);
      const int slot = 2 + 3 * parity;
      if (threadIdx.x == 0) {
        a.part[(slot + 0) * nb + blockIdx.x] = v3[0];
        a.part[(slot + 1) * nb + blockIdx.x] = v3[1];
        a.part[(slot + 2) * nb + blockIdx.x] = v3[2];
      }
      if (!grid_barrier(a.bar, a.status, a.spin)) return;
      // the scalar recurrences run once per block (thread 0) and are
      // broadcast: FP64 work is paid per warp instruction, so redundant
      // per-thread scalar math would cost as much as the vector updates.
      __shared__ double s_ab[3];
      __shared__ int s_stop;
      {
        double t3[3];
        grid_totals<3>(a.part, slot, t3);
        if (threadIdx.x == 0) {
          const double gamma = t3[0], delta = t3[1];
          rho = t3[2];
          const int stop = (rho <= a.tol2 * bnorm2 || it >= a.itmax) ? 1 : 0;
          double alpha = 0.0, beta = 0.0;
          if (!stop) {
            if (first) {
              alpha = gamma / delta;
            } else {
              beta = gamma / gamma_old;
              alpha = gamma / (delta - beta * gamma / alpha_old);
            }
            gamma_old = gamma;
            alpha_old = alpha;
          }
          s_ab[0] = alpha;
          s_ab[1] = beta;
          s_ab[2] = rho;
          s_stop = stop;
        }
        __syncthreads();
      }
      const int stop = s_stop;
      const double alpha = s_ab[0], beta = s_ab[1];
      rho = s_ab[2];
      __syncthreads();
      if (stop) break;
      first = false;
      double nv[R];
      row_apply<R>(rr, a, mb, m, nv);
#pragma unroll
      for (int k = 0; k < R; ++k) {
        if (it == it_first) {
          z[k] = nv[k]; q[k] = m[k]; s[k] = w[k]; p[k] = u[k];
        } else {
          z[k] = nv[k] + beta * z[k];
          q[k] = m[k] + beta * q[k];
          s[k] = w[k] + beta * s[k];
          p[k] = u[k] + beta * p[k];
        }
        x[k] += alpha * p[k];
        r[k] -= alpha * s[k];
        u[k] -= alpha * q[k];
        w[k] -= alpha * z[k];
      }
      parity ^= 1;
      ++it;
    }
    // publish x for the explicit residual of the next attempt
#pragma unroll
    for (int k = 0; k < R; ++k)
      if (rr.i[k] < n) a.x[rr.i[k]] = x[k];
    if (!grid_barrier(a.bar, a.status, a.spin)) return;
  }
#pragma unroll
  for (int k = 0; k < R; ++k)
    if (rr.i[k] < n) a.x[rr.i[k]] = x[k];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *a.out_iters = it;
    a.out_d[0] = rtrue2;
    a.out_d[1] = bnorm2;
    a.out_d[2] = rtrue2;
    count_solve(a.counters, it, rtrue2, bnorm2, rtrue2, a.tol2);
  }
}

int g_pcg_blocks_per_sm = -1;
int g_reg_blocks_per_sm[2] = {-1, -1};

}  // namespace

int lv_solver_assemble(lv_ctx* c, double dt) {
  if (!c->meshed) return lv_fail(c, LV_ERR_NOT_MESHED, "the grid has not been meshed");
  const int n = c->n;
  cudaStream_t s = c->stream;
  if (n > lv_fcg_capacity(c))
    if (int rc = lv_big_prepare(c)) return rc;
  c->big_masks_valid = false;
  KernelTimer kt(c, LV_KF_RHS);
  int rc = lv_scan_int(c, c->m.nfaces, c->sv.rowptr, n);
  if (rc) return rc;
  double* hr = c->sv.tmp + 2 * (size_t)c->cap;  // scratch past the scan sums
  // singular operator <=> every diagonal term is zero (c2 = Inf everywhere)
  k_half_rho<<<lv_blocks(n, TPB), TPB, 0, s>>>(c->s.rho, hr, n, c->sv.iters + LV_IT_NONSINGULAR);
  LV_LAUNCH_CHECK(c, "k_half_rho");
  k_assemble<<<lv_blocks(n, TPB), TPB, 0, s>>>(c->s, c->m, c->sv, n, dt, hr, c->sv.iters + LV_IT_NONSINGULAR);
  LV_LAUNCH_CHECK(c, "k_assemble");
  c->op_ready = true;
  c->factor_valid = false;
  return LV_OK;
}

int lv_solver_apply(lv_ctx* c, const double* x_dev, double* y_dev) {
  if (!c->op_ready) return lv_fail(c, LV_ERR_NOT_MESHED, "the pressure operator has not been assembled");
  k_spmv<<<lv_blocks(c->n, TPB), TPB, 0, c->stream>>>(c->n, c->sv.rowptr, c->sv.col, c->sv.w, c->sv.adiag, x_dev,
                                                      y_dev);
  LV_LAUNCH_CHECK(c, "k_spmv");
  return LV_OK;
}

// ---------------------------------------------------------------- sweep guess
//
// find_pressure's sweeps solve A P_k = b_k with the same operator and a
// right-hand side that follows P.  Each sweep starts from P + c1 d1 + c2 D
// (lv_sweep_sums computes c1, c2 on the right-hand side's pass); every sweep
// saves P and b for the next one, and the change P - pprev of the sweep
// before it.

// store <- P - prev (the last sweep's change; store may be nullptr); with
// shift: P <- P + c1 (P - prev) + c2 D; then prev <- P, bprev <- b (the
// values before the shift)
__global__ void k_sweep_apply(int n, double* P, double* prev, double* bprev, const double* __restrict__ b,
                              const float* __restrict__ D, float* store, const double* coef, int shift) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double p = P[i], pv = prev[i];
  if (store) store[i] = (float)(p - pv);
  if (shift) P[i] = sweep_shift(p, pv, D ? (double)D[i] : 0.0, coef[0], coef[1]);
  prev[i] = p;
  bprev[i] = b[i];
}

// store <- P - prev after the last sweep of a call
__global__ void k_sweep_store(int n, const double* __restrict__ P, const double* __restrict__ prev, float* store) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) store[i] = (float)(P[i] - prev[i]);
}

// queues the start of sweep `it` for the next solve of P (lv_solver_solve
// applies it: the flag-reduced solver inside its first residual, the other
// solvers through k_sweep_apply)
int lv_solver_sweep_guess(lv_ctx* c, double* P, int it, const float* D, float* store) {
  if (!c->op_ready) return lv_fail(c, LV_ERR_NOT_MESHED, "the pressure operator has not been assembled");
  if (int rc = lv_solver_flush_shift(c)) return rc;
  c->sg_pending = true;
  c->sg_shift = (it >= 2 || D) ? 1 : 0;
  c->sg_P = P;
  c->sg_D = D;
  c->sg_store = store;
  return LV_OK;
}

int lv_solver_flush_shift(lv_ctx* c) {
  if (!c->sg_pending) return LV_OK;
  c->sg_pending = false;
  k_sweep_apply<<<lv_blocks(c->n, TPB), TPB, 0, c->stream>>>(c->n, c->sg_P, c->sv.pprev, c->sv.bprev, c->sv.b,
                                                             c->sg_D, c->sg_store, c->sv.sgomega, c->sg_shift);
  LV_LAUNCH_CHECK(c, "k_sweep_apply");
  return LV_OK;
}

int lv_solver_sweep_store(lv_ctx* c, const double* P, float* store) {
  if (int rc = lv_solver_flush_shift(c)) return rc;
  k_sweep_store<<<lv_blocks(c->n, TPB), TPB, 0, c->stream>>>(c->n, P, c->sv.pprev, store);
  LV_LAUNCH_CHECK(c, "k_sweep_store");
  return LV_OK;
}

// Solves A x = sv.b in place in `x` (warm start = its current content) and
// stores the statistics of this solve in stats slot `slot` on the device.
int lv_solver_solve(lv_ctx* c, double* x, lv_solve_stats*, int slot) {
  if (!c->op_ready) return lv_fail(c, LV_ERR_NOT_MESHED, "the pressure operator has not been assembled");
  if (g_pcg_blocks_per_sm < 0) {
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_pcg, CG_TPB, 0);
    g_pcg_blocks_per_sm = nb > 0 ? nb : 1;
  }
  const int n = c->n;
  int maxb = c->num_sms * std::min(g_pcg_blocks_per_sm, 2);
  int nblk = std::max(1, std::min(maxb, lv_blocks(n, CG_TPB)));
  PCGArgs a;
  a.n = n;
  a.rowptr = c->sv.rowptr;
  a.col = c->sv.col;
  a.w = c->sv.w;
  a.adiag = c->sv.adiag;
  a.dinv = c->sv.dinv;
  a.b = c->sv.b;
  a.x = x;
  a.r = c->sv.r;
  a.z = c->sv.z;
  a.p = c->sv.p;
  a.q = c->sv.q;
  a.part = c->sv.part;
  a.bar = c->sv.bar;
  a.status = c->status;
  a.tol2 = c->tol * c->tol;
  a.itmax = c->itmax;
  a.spin = c->spin_limit;
  a.nonsingular = c->sv.iters + LV_IT_NONSINGULAR;
  a.diag = c->sv.diag;
  a.out_iters = c->sv.iters + slot;
  a.out_d = c->sv.dstats + 3 * slot;
  a.counters = c->sv.counters;
  if (c->method == LV_METHOD_LEARNED_PCG && !c->factor_valid) {
    // the network's factor for this operator (once per assembly)
    KernelTimer kf(c, LV_KF_LEARN);
    if (int rc = lv_learn_factor_current(c)) return rc;
    if (int rc = lv_fcg_build_minv(c)) return rc;
    c->factor_valid = true;
  }
  // a queued sweep start of x: the mixed-precision solvers apply it themselves
  const bool fcg_path = c->method == LV_METHOD_MIXED_IR || c->method == LV_METHOD_LEARNED_PCG;
  if (c->sg_pending && (!fcg_path || c->sg_P != x)) {
    KernelTimer ks(c, LV_KF_RHS);
    if (int rc = lv_solver_flush_shift(c)) return rc;
  }
  KernelTimer kt(c, LV_KF_PCG);
  if (c->method == LV_METHOD_MINRES) return lv_minres_solve(c, x, slot);
  if (c->method != LV_METHOD_JACOBI_PCG) {
    const bool learned = c->method == LV_METHOD_LEARNED_PCG;
    // systems that fit one or two blocks per SM: flag-reduced solver
    if (n <= lv_fcg_capacity(c)) return lv_fcg_solve(c, x, slot, learned);  // applies a queued start of x itself
    // larger systems: the streaming variant
    return lv_big_solve(c, x, slot, learned);
  }
  cudaMemsetAsync(c->sv.bar, 0, 2 * sizeof(unsigned), c->stream);
  // small systems: register-resident pipelined CG, one barrier per iteration
  if (g_reg_blocks_per_sm[0] < 0) {
    int b1 = 0, b2 = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b1, k_pcg_reg<1>, SP_TPB, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b2, k_pcg_reg<2>, SP_TPB, 0);
    g_reg_blocks_per_sm[0] = b1;
    g_reg_blocks_per_sm[1] = b2;
  }
  for (int R = 1; R <= 2; ++R) {
    const int per_sm = std::min(g_reg_blocks_per_sm[R - 1], 2);
    if (per_sm < 1) continue;
    const int cap_blocks = c->num_sms * per_sm;
    const int need = lv_blocks(n, SP_TPB * R);
    if (need > cap_blocks) continue;
    double* ubuf = c->sv.tmp;
    double* mb0 = c->sv.tmp + c->cap;
    double* mb1 = c->sv.r + c->cap;  // second half of r (2*cap doubles)
    void* rargs[] = {&a, &ubuf, &mb0, &mb1};
    const void* fn = (R == 1) ? (const void*)k_pcg_reg<1> : (const void*)k_pcg_reg<2>;
    cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(std::max(need, 1)), dim3(SP_TPB), rargs, 0, c->stream);
    c->launches++;
    if (e != cudaSuccess) return lv_cuda_check(c, e, "k_pcg_reg cooperative launch");
    return LV_OK;
  }
  void* args[] = {&a};
  cudaError_t e = cudaLaunchCooperativeKernel((const void*)k_pcg, dim3(nblk), dim3(CG_TPB), args, 0, c->stream);
  c->launches++;
  if (e != cudaSuccess) return lv_cuda_check(c, e, "k_pcg cooperative launch");
  return LV_OK;
}

int lv_solver_fetch_stats(lv_ctx* c, lv_solve_stats* out, int count) {
  std::vector<int> it(count), outer(count), meth(count);
  std::vector<double> d(3 * count);
  cudaMemcpyAsync(meth.data(), c->sv.iters + LV_IT_METHOD, sizeof(int) * count, cudaMemcpyDeviceToHost, c->stream);
  cudaMemcpyAsync(outer.data(), c->sv.iters + LV_IT_OUTER, sizeof(int) * count, cudaMemcpyDeviceToHost, c->stream);
  cudaMemcpyAsync(it.data(), c->sv.iters, sizeof(int) * count, cudaMemcpyDeviceToHost, c->stream);
  cudaMemcpyAsync(d.data(), c->sv.dstats, sizeof(double) * 3 * count, cudaMemcpyDeviceToHost, c->stream);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return lv_cuda_check(c, e, "fetch stats");
  for (int k = 0; k < count; ++k) {
    const double rr = d[3 * k], bb = d[3 * k + 1], tr = d[3 * k + 2];
    out[k].iterations = it[k];
    if (c->method == LV_METHOD_MINRES) {
      // MINRES's own stopping tests (absolute + relative, least squares)
      out[k].converged = outer[k] != 0 ? 1 : 0;
      out[k].outer = 0;
      out[k].method = LV_METHOD_MINRES;
    } else {
      out[k].converged = (rr <= c->tol * c->tol * bb) ? 1 : 0;
      out[k].outer = c->method == LV_METHOD_JACOBI_PCG ? 0 : outer[k];
      out[k].method = c->method == LV_METHOD_JACOBI_PCG ? c->method : meth[k];
    }
    out[k].rel_residual = bb > 0 ? sqrt(tr / bb) : sqrt(tr);
  }
  return LV_OK;
}

// ===================================================================
// Allocation-free solve (lv_pcg_solve_noalloc).
//
// Callers that cannot allocate device memory still get the FP64
// Jacobi-PCG: the kernel's scratch lives in the file-scope array below
// instead of buffers from cudaMalloc.  The array is sized for
// LV_NOALLOC_MAX_ROWS rows and every GPU that loads this library keeps it
// (about 24 MiB) until the process exits.  All calls share it, and it keeps
// the contents of the last call.  Two calls that overlap on the GPU race on
// it.
// ===================================================================

namespace {

constexpr int NOALLOC_VECS = 6;                   // adiag, dinv, r, z, p, q
constexpr int NOALLOC_PART = 4 * 4096;            // reduction partials
constexpr int NOALLOC_MISC = 64;                  // barrier, flags, statistics
constexpr size_t NOALLOC_DOUBLES = (size_t)NOALLOC_VECS * LV_NOALLOC_MAX_ROWS + NOALLOC_PART + NOALLOC_MISC;

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_DOUBLES];

// adiag_i = diag_i + sum_j w_ij, dinv_i = 1/adiag_i, and the flag telling
// whether any diagonal term is nonzero (nonsingular operator).
__global__ void k_noalloc_diag(int n, const double* __restrict__ diag, const int* __restrict__ rowptr,
                               const double* __restrict__ w, double* adiag, double* dinv, int* nonsingular) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double d = diag[i];
  double ad = d;
  for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) ad += w[k];
  adiag[i] = ad;
  dinv[i] = 1.0 / ad;
  if (d != 0.0) atomicOr(nonsingular, 1);
}

// Device address of the scratch array, looked up once per device (by the
// first call on that device, whichever host thread makes it).
double* g_noalloc_dev[LV_MAX_DEVICES] = {nullptr};
std::once_flag g_noalloc_once[LV_MAX_DEVICES];

}  // namespace

extern "C" int lv_pcg_solve_noalloc(int32_t n, const double* diag, const int32_t* rowptr, const int32_t* col,
                                    const double* w, const double* b, double* x, double tol, int32_t itmax,
                                    void* stream, int32_t* iterations, double* rel_residual) {
  if (n <= 0 || n > LV_NOALLOC_MAX_ROWS) return LV_ERR_BAD_ARGUMENT;
  if (!diag || !rowptr || !col || !w || !b || !x || !(tol > 0) || itmax <= 0) return LV_ERR_BAD_ARGUMENT;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= LV_MAX_DEVICES) return LV_ERR_CUDA;
  // First call on this device: resolve the array's device address with the
  // device current.  The host-side name g_noalloc_scratch is only a stand-in
  // and must never be passed to a kernel.
  std::call_once(g_noalloc_once[dev], [dev]() {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) == cudaSuccess) g_noalloc_dev[dev] = static_cast<double*>(p);
  });
  double* base = g_noalloc_dev[dev];
  if (!base) return LV_ERR_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t M = LV_NOALLOC_MAX_ROWS;
  double* adiag = base;
  double* dinv = base + M;
  double* misc = base + NOALLOC_VECS * M + NOALLOC_PART;
  unsigned* bar = reinterpret_cast<unsigned*>(misc);          // 2 words
  int* status = reinterpret_cast<int*>(misc + 1);
  int* nonsingular = reinterpret_cast<int*>(misc + 2);
  int* iters = reinterpret_cast<int*>(misc + 3);
  double* outd = misc + 4;                                     // rr, bb, true rr
  long long* counters = reinterpret_cast<long long*>(misc + 8);  // 3 words
  // what must start at zero: barrier, status, flag, counters
  if (cudaMemsetAsync(misc, 0, sizeof(double) * 11, s) != cudaSuccess) return LV_ERR_CUDA;
  k_noalloc_diag<<<lv_blocks(n, TPB), TPB, 0, s>>>(n, diag, rowptr, w, adiag, dinv, nonsingular);
  if (cudaGetLastError() != cudaSuccess) return LV_ERR_CUDA;
  int sms = 0, per_sm = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return LV_ERR_CUDA;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg, CG_TPB, 0) != cudaSuccess || per_sm < 1)
    return LV_ERR_CUDA;
  const int nblk = std::max(1, std::min(sms * std::min(per_sm, 2), lv_blocks(n, CG_TPB)));
  PCGArgs a;
  a.n = n;
  a.rowptr = rowptr;
  a.col = col;
  a.w = w;
  a.adiag = adiag;
  a.dinv = dinv;
  a.b = b;
  a.x = x;
  a.r = base + 2 * M;
  a.z = base + 3 * M;
  a.p = base + 4 * M;
  a.q = base + 5 * M;
  a.part = base + NOALLOC_VECS * M;
  a.bar = bar;
  a.status = status;
  a.tol2 = tol * tol;
  a.itmax = itmax;
  a.spin = LV_WAIT_LIMIT_DEFAULT;
  a.nonsingular = nonsingular;
  a.diag = diag;
  a.out_iters = iters;
  a.out_d = outd;
  a.counters = counters;
  void* args[] = {&a};
  if (cudaLaunchCooperativeKernel((const void*)k_pcg, dim3(nblk), dim3(CG_TPB), args, 0, s) != cudaSuccess)
    return LV_ERR_CUDA;
  if (!iterations && !rel_residual) return LV_OK;
  int it = 0, st = 0;
  double d3[3] = {0, 0, 0};
  if (cudaMemcpyAsync(&it, iters, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(&st, status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(d3, outd, sizeof(d3), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return LV_ERR_CUDA;
  if (st & LV_FLAG_BARRIER_TIMEOUT) return LV_ERR_BARRIER_TIMEOUT;
  if (iterations) *iterations = it;
  if (rel_residual) *rel_residual = d3[1] > 0 ? sqrt(d3[2] / d3[1]) : sqrt(d3[2]);
  // both the recursive residual (the loop's test) and the true one recomputed
  // at the end must meet the tolerance
  return (d3[0] <= tol * tol * d3[1] && d3[2] <= tol * tol * d3[1]) ? LV_OK : LV_ERR_CG_MAXITER;
}
