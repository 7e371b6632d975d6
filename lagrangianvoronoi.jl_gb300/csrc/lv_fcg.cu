// Mixed-precision pressure solve (LV_METHOD_MIXED_IR and LV_METHOD_LEARNED_PCG)
// for systems whose rows fit the registers of one block per SM.
//
// The operator is the reference's PressureOperator (pressure.jl:89-130):
//   (A x)_i = diag_i x_i + sum_j w_ij (x_i - x_j).
// x and the true residual b - A x (that difference form, exact on constants)
// are FP64 and checked against tol ||b||.  In between, preconditioned CG runs
// in FP32 on the residual scaled to unit norm; each refinement step folds
// the FP32 correction into x and restarts from the FP64 residual (k_fcg).  The preconditioner is Jacobi or the learned
// M^-1 = D^-1/2 (Gt^T Gt + eps I) D^-1/2 (Gt from lv_learn.cu), held as an
// explicit sparse matrix on the two-hop pattern of the operator so that
// applying it needs one neighbour exchange.
//
// Synchronisation: dot products travel through grid-wide phases (fphase: each
// block publishes its partial sums and one arrival; every block sums all
// partials in the same fixed order); neighbour values through point-to-point
// exchanges (nexchange: per-block flags, each block waits only for the blocks
// whose rows it reads).  A Jacobi iteration costs one exchange and one phase,
// a learned one two exchanges and one phase.
#include "lv_internal.cuh"

namespace {

constexpr int FCG_TPB = 512;
constexpr int FCG_NW = FCG_TPB / 32;
constexpr int FKR = 8;    // operator entries per row held in registers
constexpr int FKM = 12;   // preconditioner off-diagonal entries per row held in registers
constexpr int MMAX = 96;  // preconditioner off-diagonal entries per row (storage slots)
constexpr long long FCG_SPIN_LIMIT = 4000000000LL;  // cycles (about 2 s)
constexpr float FCG_UPDATE_DROP = 1e-5f;  // FP32 residual reduction per refinement step
constexpr int FCG_MAX_UPDATES = 200;

constexpr int RG_WORDS = 4;  // partial-sum words per block and phase
constexpr int FLAG_STRIDE = 32;  // exchange flags sit on separate 128-byte lines (packed flags halve the speed)
constexpr int FCG_MAX_BLOCKS = 1024;

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

struct FcgArgs {
  int n, nb, rows_per_block;
  const int* rowptr;
  const int* col;
  const double* w;
  const double* diag;  // the reference's diagonal term (mass part)
  const double* dinv;  // 1 / (diag + sum_j w_ij)
  const double* b;
  double* x;  // FP64 iterate, also the exchange buffer of the outer residual
  float* rbuf;
  float* ubuf;    // u exchange
  unsigned long long* slots;  // partial words [2 parities][RG_WORDS][nb] (as 32-bit words)
  unsigned* counter;          // arrivals, zeroed before the launch
  unsigned* flags;            // per-block exchange epochs, one 128-byte line each (FLAG_STRIDE words)
  int* status;
  double tol2;
  int itmax;
  const int* nonsingular;
  int learned;
  const int* mcnt;  // learned M^-1: off-diagonal count, slot-major entries, diagonal
  const int* mcol;
  const float* mval;
  const float* mdiag;
  int mstride;
  const int* minv_ok;
  int* jref;
  int* out_iters;
  int* out_outer;
  int* out_method;
  double* out_d;
  long long* counters;
};

// One phase: publish this block's NV partial sums and sum all blocks'
// partials (T = float for the inner solve, double for the FP64 outer loop).
// Each block stores its words (double-buffered by phase parity), then
// increments one arrival counter with release semantics; thread 0 waits until
// the counter reaches phase x blocks, and the block reads every block's words
// once.  The phase is both a grid-wide synchronisation (values stored before
// it are visible after it) and the reduction, summed in a fixed order, so
// every block holds bit-identical totals.
__device__ __forceinline__ void red_release_add(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// thread 0: arrive and wait for phase ph; returns 0 on timeout
__device__ __forceinline__ int arrive_wait(const FcgArgs& a, unsigned ph) {
  red_release_add(a.counter, 1u);
  const unsigned target = ph * (unsigned)a.nb;
  const long long t0 = clock64();
  while (ld_acquire_u32(a.counter) < target) {
    if (clock64() - t0 > FCG_SPIN_LIMIT) {
      atomicOr(a.status, LV_FLAG_BARRIER_TIMEOUT);
      return 0;
    }
  }
  return 1;
}

template <typename T>
__device__ __forceinline__ T allsum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename T>
struct Words;
template <>
struct Words<float> {
  static constexpr int N = 1;
  __device__ static void put(float v, unsigned* w) { w[0] = __float_as_uint(v); }
  __device__ static float get(const unsigned* w) { return __uint_as_float(w[0]); }
};
template <>
struct Words<double> {
  static constexpr int N = 2;
  __device__ static void put(double v, unsigned* w) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(v);
    w[0] = (unsigned)(u >> 32);
    w[1] = (unsigned)u;
  }
  __device__ static double get(const unsigned* w) {
    return __longlong_as_double((long long)(((unsigned long long)w[0] << 32) | w[1]));
  }
};

template <int NV, typename T>
__device__ bool fphase(const FcgArgs& a, unsigned ph, const T (&v)[NV], T (&tot)[NV]) {
  constexpr int NWD = NV * Words<T>::N;
  static_assert(NWD <= RG_WORDS, "at most four words per block");
  __shared__ T shw[NV * 32];
  __shared__ T shw2[NV * 32];
  __shared__ int s_ok;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned* words = reinterpret_cast<unsigned*>(a.slots) + (size_t)(ph & 1u) * RG_WORDS * a.nb;
  // 1. this block's partials
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const T t = allsum(v[k]);
    if (lane == 0) shw[k * 32 + wid] = t;
  }
  __syncthreads();
  if (wid == 0) {
    unsigned wd[NWD];
#pragma unroll
    for (int k = 0; k < NV; ++k) Words<T>::put(allsum(lane < FCG_NW ? shw[k * 32 + lane] : T(0)), wd + k * Words<T>::N);
    if (lane == 0) {
#pragma unroll
      for (int q = 0; q < NWD; ++q) __stcg(words + (size_t)q * a.nb + blockIdx.x, wd[q]);
      s_ok = arrive_wait(a, ph);
    }
  }
  __syncthreads();
  if (!s_ok) return false;
  // 2. every block's words, read once: thread t reads block t's
  T acc[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) acc[k] = T(0);
  if ((int)threadIdx.x < a.nb) {
    unsigned wd[NWD];
#pragma unroll
    for (int q = 0; q < NWD; ++q) wd[q] = __ldcg(words + (size_t)q * a.nb + threadIdx.x);
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = Words<T>::get(wd + k * Words<T>::N);
  }
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    acc[k] = allsum(acc[k]);
    if (lane == 0) shw2[k * 32 + wid] = acc[k];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    T t = T(0);
#pragma unroll
    for (int q = 0; q < FCG_NW; ++q) t += shw2[k * 32 + q];
    tot[k] = t;
  }
  return true;
}

__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Neighbour exchange number e: the values this block stored before it are
// visible to the blocks that read them, and this block sees the values of
// the blocks in its mask (the owners of the columns its rows reference).
// Point to point: each block raises its own flag and waits only for its
// neighbours' flags.  Consecutive exchanges are always separated by a
// grid-wide phase, so one buffer per exchanged vector suffices.
__device__ bool nexchange(const FcgArgs& a, unsigned e, const unsigned* mask) {
  __syncthreads();
  if (threadIdx.x == 0) st_release_u32(a.flags + (size_t)blockIdx.x * FLAG_STRIDE, e);
  int to = 0;
  const int t = threadIdx.x;
  if (t < a.nb && ((mask[t >> 5] >> (t & 31)) & 1u)) {
    const long long t0 = clock64();
    while (ld_acquire_u32(a.flags + (size_t)t * FLAG_STRIDE) < e) {
      if (clock64() - t0 > FCG_SPIN_LIMIT) {
        to = 1;
        atomicOr(a.status, LV_FLAG_BARRIER_TIMEOUT);
        break;
      }
    }
  }
  return __syncthreads_or(to) == 0;
}

template <int R>
struct FRows {
  int i[R];
  bool on[R];
  int beg[R], cnt[R];
  int cc[R][FKR];
  float ww[R][FKR];
  float dg[R], dnv[R];
  int mn[R];
  int mc[R][FKM];
  float mv[R][FKM];
  float md[R];
  double bb[R];
};

template <int R>
__global__ void __launch_bounds__(FCG_TPB, 1) k_fcg(FcgArgs a) {
  const int n = a.n;
  const int rb0 = blockIdx.x * a.rows_per_block;
  const int rb1 = min(n, rb0 + a.rows_per_block);
  const bool learned0 = a.learned != 0 && *a.minv_ok != 0;
  FRows<R> rr;
  double x[R];
#pragma unroll
  for (int k = 0; k < R; ++k) {
    const int i = rb0 + (int)threadIdx.x + k * FCG_TPB;
    const bool on = i < rb1;
    rr.i[k] = i;
    rr.on[k] = on;
    rr.beg[k] = on ? a.rowptr[i] : 0;
    rr.cnt[k] = on ? a.rowptr[i + 1] - rr.beg[k] : 0;
#pragma unroll
    for (int e = 0; e < FKR; ++e) {
      const bool have = e < rr.cnt[k];
      rr.cc[k][e] = have ? a.col[rr.beg[k] + e] : 0;
      rr.ww[k][e] = have ? (float)a.w[rr.beg[k] + e] : 0.f;
    }
    rr.dg[k] = on ? (float)a.diag[i] : 0.f;
    rr.dnv[k] = on ? (float)a.dinv[i] : 0.f;
    rr.mn[k] = (on && learned0) ? a.mcnt[i] : 0;
#pragma unroll
    for (int e = 0; e < FKM; ++e) {
      const bool have = e < rr.mn[k];
      rr.mc[k][e] = have ? a.mcol[(size_t)e * a.mstride + i] : 0;
      rr.mv[k][e] = have ? a.mval[(size_t)e * a.mstride + i] : 0.f;
    }
    rr.md[k] = (on && learned0) ? a.mdiag[i] : 0.f;
    rr.bb[k] = on ? a.b[i] : 0.0;
    x[k] = on ? a.x[i] : 0.0;
  }
  // blocks owning the columns of this block's rows (operator and M^-1)
  __shared__ unsigned s_mask[FCG_MAX_BLOCKS / 32];
  for (int t = threadIdx.x; t < FCG_MAX_BLOCKS / 32; t += FCG_TPB) s_mask[t] = 0u;
  __syncthreads();
  {
    const int rpb = a.rows_per_block;
    const int me = blockIdx.x;
    auto mark = [&](int j) {
      const int bj = j / rpb;
      if (bj != me) atomicOr(&s_mask[bj >> 5], 1u << (bj & 31));
    };
#pragma unroll
    for (int k = 0; k < R; ++k) {
      if (!rr.on[k]) continue;
      for (int e = rr.beg[k]; e < rr.beg[k] + rr.cnt[k]; ++e) mark(a.col[e]);
      for (int e = 0; e < rr.mn[k]; ++e) mark(a.mcol[(size_t)e * a.mstride + rr.i[k]]);
    }
  }
  unsigned ep = 0;  // phases completed in this launch
  unsigned xe = 0;  // neighbour exchanges completed in this launch
  bool ok = true;
  // singular operator: project b to zero mean
  if (*a.nonsingular == 0) {
    double v[1] = {0.0}, t[1];
#pragma unroll
    for (int k = 0; k < R; ++k) v[0] += rr.bb[k];
    ok = fphase<1, double>(a, ++ep, v, t);
    const double mean = t[0] / (double)n;
#pragma unroll
    for (int k = 0; k < R; ++k)
      if (rr.on[k]) rr.bb[k] -= mean;
  }
  const int jref = *a.jref;
  const int cap = jref > 0 ? jref : a.itmax;
  bool learned = learned0;
  int it = 0, updates = 0;
  double bnorm2 = 0.0, rtrue2 = 0.0;
  float r[R], u[R], w[R], p[R], s[R], d[R];
  // out = A v with the neighbours' values from buf (FP32 difference form)
  auto spmv = [&](const float* buf, const float(&own)[R], float(&out)[R]) {
#pragma unroll
    for (int k = 0; k < R; ++k) {
      float acc = rr.dg[k] * own[k];
#pragma unroll
      for (int e = 0; e < FKR; ++e)
        if (e < rr.cnt[k]) acc = fmaf(rr.ww[k][e], own[k] - __ldcg(buf + rr.cc[k][e]), acc);
      for (int e = FKR; e < rr.cnt[k]; ++e)
        acc = fmaf((float)a.w[rr.beg[k] + e], own[k] - __ldcg(buf + a.col[rr.beg[k] + e]), acc);
      out[k] = acc;
    }
  };
  // out = M^-1 v (learned) with the neighbours' values from buf
  auto mapply = [&](const float* buf, const float(&own)[R], float(&out)[R]) {
#pragma unroll
    for (int k = 0; k < R; ++k) {
      float t = rr.md[k] * own[k];
#pragma unroll
      for (int e = 0; e < FKM; ++e)
        if (e < rr.mn[k]) t = fmaf(rr.mv[k][e], __ldcg(buf + rr.mc[k][e]), t);
      for (int e = FKM; e < rr.mn[k]; ++e) {
        const size_t q = (size_t)e * a.mstride + rr.i[k];
        t = fmaf(a.mval[q], __ldcg(buf + a.mcol[q]), t);
      }
      out[k] = t;
    }
  };
  // u = M^-1 r (the learned preconditioner needs r from the neighbours)
  auto precond = [&]() -> bool {
    if (learned) {
#pragma unroll
      for (int k = 0; k < R; ++k)
        if (rr.on[k]) a.rbuf[rr.i[k]] = r[k];
      if (!nexchange(a, ++xe, s_mask)) return false;
      mapply(a.rbuf, r, u);
    } else {
#pragma unroll
      for (int k = 0; k < R; ++k) u[k] = rr.dnv[k] * r[k];
    }
    return true;
  };
  // FP32 CG on A d = r / sigma, single-reduction form (Chronopoulos & Gear,
  // J. Comput. Appl. Math. 25, 1989; D'Azevedo, Eijkhout & Romine, LAPACK
  // Working Note 56, 1993): gamma = (r, u), delta = (A u, u) and ||r||^2 in
  // one grid-wide phase, alpha = gamma / (delta - beta gamma / alpha_old);
  // u = M^-1 r and w = A u are computed directly each iteration (only s = A p
  // is a recurrence), their neighbour values moved by point-to-point
  // exchanges.  Iterative refinement: once the FP32 residual has dropped by
  // FCG_UPDATE_DROP, or the target is in reach, x += sigma d in FP64, the
  // residual is recomputed in FP64 (difference form) and CG restarts on it.
  // (Continuing the old directions across the replacement instead breaks the
  // orthogonality the single-reduction alpha relies on, and stalled on the
  // singular operators of incompressible flows.)
  double sigma = 1.0;
  bool have_d = false, first = true, fall = false;
  float gam_old = 1.f, alpha = 1.f;
  while (ok) {
    if (have_d) {
#pragma unroll
      for (int k = 0; k < R; ++k) {
        x[k] += sigma * (double)d[k];
        if (rr.on[k]) a.x[rr.i[k]] = x[k];
      }
      if (!(ok = nexchange(a, ++xe, s_mask))) break;
    }
    double r64[R];
    double v[2] = {0.0, 0.0}, t2[2];
#pragma unroll
    for (int k = 0; k < R; ++k) {
      double acc = 0.0;
      if (rr.on[k]) {
        acc = a.diag[rr.i[k]] * x[k];
        for (int e = rr.beg[k]; e < rr.beg[k] + rr.cnt[k]; ++e) acc += a.w[e] * (x[k] - __ldcg(a.x + a.col[e]));
      }
      r64[k] = rr.on[k] ? rr.bb[k] - acc : 0.0;
      v[0] += r64[k] * r64[k];
      v[1] += rr.bb[k] * rr.bb[k];
    }
    if (!(ok = fphase<2, double>(a, ++ep, v, t2))) break;
    rtrue2 = t2[0];
    bnorm2 = t2[1];
    if (rtrue2 <= a.tol2 * bnorm2 || it >= a.itmax || updates >= FCG_MAX_UPDATES) break;
    sigma = sqrt(rtrue2);
    const double inv_sigma = 1.0 / sigma;
#pragma unroll
    for (int k = 0; k < R; ++k) {
      r[k] = (float)(r64[k] * inv_sigma);
      d[k] = 0.f;
    }
    have_d = true;
    ++updates;
    first = true;  // CG restarts from the refined iterate
    if (fall) {
      // the learned preconditioner needed more iterations than Jacobi did:
      // continue from the current iterate with Jacobi
      learned = false;
      fall = false;
    }
    const float rho_upd = fmaxf(FCG_UPDATE_DROP * FCG_UPDATE_DROP, (float)(0.25 * a.tol2 * bnorm2 / rtrue2));
    if (!(ok = precond())) break;
    while (true) {
#pragma unroll
      for (int k = 0; k < R; ++k)
        if (rr.on[k]) a.ubuf[rr.i[k]] = u[k];
      if (!(ok = nexchange(a, ++xe, s_mask))) break;
      spmv(a.ubuf, u, w);
      float v3[3] = {0.f, 0.f, 0.f}, t3[3];
#pragma unroll
      for (int k = 0; k < R; ++k) {
        v3[0] = fmaf(r[k], u[k], v3[0]);
        v3[1] = fmaf(w[k], u[k], v3[1]);
        v3[2] = fmaf(r[k], r[k], v3[2]);
      }
      if (!(ok = fphase<3, float>(a, ++ep, v3, t3))) break;
      const float gam = t3[0], delta = t3[1], rho = t3[2];
      if (rho <= rho_upd || it >= a.itmax || !(delta > 0.f)) break;
      if (learned && it >= cap) {
        fall = true;
        break;
      }
      const float beta = first ? 0.f : gam / gam_old;
      alpha = first ? gam / delta : gam / (delta - beta * gam / alpha);
#pragma unroll
      for (int k = 0; k < R; ++k) {
        p[k] = first ? u[k] : fmaf(beta, p[k], u[k]);
        s[k] = first ? w[k] : fmaf(beta, s[k], w[k]);
        d[k] = fmaf(alpha, p[k], d[k]);
        r[k] = fmaf(-alpha, s[k], r[k]);
      }
      gam_old = gam;
      first = false;
      ++it;
      if (!(ok = precond())) break;
    }
  }
  if (ok && blockIdx.x == 0 && threadIdx.x == 0) {
    *a.out_iters = it;
    *a.out_outer = updates;
    *a.out_method = learned ? LV_METHOD_LEARNED_PCG : LV_METHOD_MIXED_IR;
    if (!a.learned) *a.jref = it;
    a.out_d[0] = rtrue2;
    a.out_d[1] = bnorm2;
    a.out_d[2] = rtrue2;
    a.counters[0] += 1;
    a.counters[1] += it;
  }
}

// M^-1 = D^-1/2 (Gt^T Gt + eps I) D^-1/2, one thread per row i:
// (Gt^T Gt)_ij = sum_k Gt_ki Gt_kj over k in {i} and the rows whose pattern
// holds i (the upper neighbours of i, and with the two-hop pattern its upper
// two-hop neighbours), j over the pattern of row k (k, its lower neighbours
// and lower two-hop neighbours).  Two hops of Gt give M^-1 two (one-hop
// pattern) or four (two-hop pattern) hops.
__global__ void k_build_minv(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                             const float* __restrict__ gd, const float* __restrict__ gl, const int* __restrict__ rev,
                             const int* __restrict__ rowptr2, const int* __restrict__ col2,
                             const float* __restrict__ gl2, const int* __restrict__ rev2,
                             const float* __restrict__ dh, float eps, int stride, int* mcnt, int* mcol, float* mval,
                             float* mdiag, int* ok) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int cols[MMAX];
  float vals[MMAX];
  int m = 0;
  float dsum = 0.f;
  bool overflow = false;
  auto add = [&](int j, float v) {
    if (j == i) {
      dsum += v;
      return;
    }
    for (int s = 0; s < m; ++s)
      if (cols[s] == j) {
        vals[s] += v;
        return;
      }
    if (m < MMAX) {
      cols[m] = j;
      vals[m] = v;
      ++m;
    } else {
      overflow = true;
    }
  };
  // row k of Gt times Gt_ki
  auto row_k = [&](int k, float gki) {
    add(k, gki * gd[k]);
    for (int k2 = rowptr[k]; k2 < rowptr[k + 1]; ++k2)
      if (col[k2] < k) add(col[k2], gki * gl[k2]);
    if (rowptr2)
      for (int e = rowptr2[k]; e < rowptr2[k + 1]; ++e)
        if (col2[e] < k) add(col2[e], gki * gl2[e]);
  };
  row_k(i, gd[i]);
  for (int kk = rowptr[i]; kk < rowptr[i + 1]; ++kk) {
    const int u = col[kk];
    if (u > i && rev[kk] >= 0) row_k(u, gl[rev[kk]]);
  }
  if (rowptr2)
    for (int e = rowptr2[i]; e < rowptr2[i + 1]; ++e) {
      const int u = col2[e];
      if (u > i && rev2[e] >= 0) row_k(u, gl2[rev2[e]]);
    }
  const float di = dh[i];
  for (int s = 0; s < m; ++s) {
    mcol[(size_t)s * stride + i] = cols[s];
    mval[(size_t)s * stride + i] = di * vals[s] * dh[cols[s]];
  }
  mcnt[i] = m;
  mdiag[i] = di * (dsum + eps) * di;
  if (overflow) atomicAnd(ok, 0);
}

int g_fcg_blocks_per_sm[2] = {-1, -1};



}  // namespace

// Rows the flag-reduced solver holds (one or two blocks per SM, two rows per
// thread at most); larger systems use the streaming solver.
int lv_fcg_capacity(lv_ctx* c) {
  if (g_fcg_blocks_per_sm[0] < 0) {
    int b1 = 0, b2 = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b1, k_fcg<1>, FCG_TPB, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b2, k_fcg<2>, FCG_TPB, 0);
    g_fcg_blocks_per_sm[0] = b1;
    g_fcg_blocks_per_sm[1] = b2;
  }
  if (g_fcg_blocks_per_sm[1] < 1) return 0;
  const int per_sm = std::min(g_fcg_blocks_per_sm[1], 2);
  return std::min(c->num_sms * per_sm, FCG_MAX_BLOCKS) * FCG_TPB * 2;
}

static int ensure_minv(lv_ctx* c) {
  SolverDev& sv = c->sv;
  const int rows = std::min(c->cap, lv_fcg_capacity(c));
  if (sv.mrows >= rows && sv.mcnt) return LV_OK;
  cudaFree(sv.mcnt);
  cudaFree(sv.mcol);
  cudaFree(sv.mval);
  cudaFree(sv.mdiag);
  cudaFree(sv.mok);
  sv.mcnt = nullptr;
  sv.mcol = nullptr;
  sv.mval = nullptr;
  sv.mdiag = nullptr;
  sv.mok = nullptr;
  sv.mrows = 0;
  bool ok = cudaMalloc(&sv.mcnt, sizeof(int) * rows) == cudaSuccess;
  ok = ok && cudaMalloc(&sv.mcol, sizeof(int) * (size_t)MMAX * rows) == cudaSuccess;
  ok = ok && cudaMalloc(&sv.mval, sizeof(float) * (size_t)MMAX * rows) == cudaSuccess;
  ok = ok && cudaMalloc(&sv.mdiag, sizeof(float) * rows) == cudaSuccess;
  ok = ok && cudaMalloc(&sv.mok, sizeof(int)) == cudaSuccess;
  if (!ok) return lv_fail(c, LV_ERR_CUDA, "allocation of the learned preconditioner matrix failed");
  cudaMemsetAsync(sv.mok, 0, sizeof(int), c->stream);
  sv.mrows = rows;
  return LV_OK;
}

void lv_fcg_free(lv_ctx* c) {
  SolverDev& sv = c->sv;
  cudaFree(sv.mcnt);
  cudaFree(sv.mcol);
  cudaFree(sv.mval);
  cudaFree(sv.mdiag);
  cudaFree(sv.mok);
  sv.mcnt = nullptr;
  sv.mcol = nullptr;
  sv.mval = nullptr;
  sv.mdiag = nullptr;
  sv.mok = nullptr;
  sv.mrows = 0;
}

// Builds the explicit learned M^-1 from the current factor (after
// lv_learn_factor_current).
int lv_fcg_build_minv(lv_ctx* c) {
  const int n = c->n;
  if (n > lv_fcg_capacity(c)) return LV_OK;  // the streaming solver applies the factor itself
  if (int rc = ensure_minv(c)) return rc;
  const float *gd, *gl, *dh, *gl2;
  const int *rev, *rowptr2, *col2, *rev2;
  lv_learn_factor_ptrs(c, &gd, &gl, &dh, &rev);
  lv_learn_factor2_ptrs(c, &rowptr2, &col2, &gl2, &rev2);
  if (!gd) return lv_fail(c, LV_ERR_BAD_ARGUMENT, "learned solve without a factor");
  const int one = 1;
  cudaMemcpyAsync(c->sv.mok, &one, sizeof(int), cudaMemcpyHostToDevice, c->stream);
  k_build_minv<<<lv_blocks(n, 128), 128, 0, c->stream>>>(n, c->sv.rowptr, c->sv.col, gd, gl, rev, rowptr2, col2, gl2,
                                                          rev2, dh, c->learn_eps, c->sv.mrows, c->sv.mcnt,
                                                          c->sv.mcol, c->sv.mval, c->sv.mdiag, c->sv.mok);
  LV_LAUNCH_CHECK(c, "k_build_minv");
  return LV_OK;
}

// Launches the flag-reduced mixed-precision solve into x (device), stats into
// the given slot.  Returns LV_ERR_BAD_ARGUMENT when the system is too large.
int lv_fcg_solve(lv_ctx* c, double* x, int slot, bool learned) {
  const int n = c->n;
  const int capn = lv_fcg_capacity(c);
  if (n > capn || n < 1) return LV_ERR_BAD_ARGUMENT;
  if (learned && !c->sv.mcnt) return lv_fail(c, LV_ERR_BAD_ARGUMENT, "learned solve without a preconditioner");
  // one block per SM while one row per thread suffices, else two rows per
  // thread, then two blocks per SM
  int nb = c->num_sms, R = 1;
  if (n > nb * FCG_TPB) R = 2;
  if (n > nb * FCG_TPB * 2) nb = std::min(c->num_sms * 2, FCG_MAX_BLOCKS);
  if (g_fcg_blocks_per_sm[R - 1] * c->num_sms < nb) return LV_ERR_BAD_ARGUMENT;
  FcgArgs a;
  a.n = n;
  a.nb = nb;
  a.rows_per_block = (n + nb - 1) / nb;
  a.rowptr = c->sv.rowptr;
  a.col = c->sv.col;
  a.w = c->sv.w;
  a.diag = c->sv.diag;
  a.dinv = c->sv.dinv;
  a.b = c->sv.b;
  a.x = x;
  a.rbuf = c->sv.r32;
  a.ubuf = c->sv.f32a;
  a.slots = c->sv.fslots;
  a.counter = c->sv.bar + 2;
  a.flags = reinterpret_cast<unsigned*>(c->sv.fslots + 8192);
  a.status = c->status;
  a.tol2 = c->tol * c->tol;
  a.itmax = c->itmax;
  a.nonsingular = c->sv.iters + LV_IT_NONSINGULAR;
  a.learned = learned ? 1 : 0;
  a.mcnt = c->sv.mcnt;
  a.mcol = c->sv.mcol;
  a.mval = c->sv.mval;
  a.mdiag = c->sv.mdiag;
  a.mstride = c->sv.mrows;
  a.minv_ok = learned ? c->sv.mok : c->sv.iters + LV_IT_NONSINGULAR;  // read only in learned mode
  a.jref = c->sv.iters + LV_IT_JREF + slot;  // the same sweep of the last Jacobi mixed solve
  a.out_iters = c->sv.iters + slot;
  a.out_outer = c->sv.iters + LV_IT_OUTER + slot;
  a.out_method = c->sv.iters + LV_IT_METHOD + slot;
  a.out_d = c->sv.dstats + 3 * slot;
  a.counters = c->sv.counters;
  cudaMemsetAsync(c->sv.bar + 2, 0, sizeof(unsigned), c->stream);
  cudaMemsetAsync(a.flags, 0, sizeof(unsigned) * FLAG_STRIDE * nb, c->stream);
  void* args[] = {&a};
  const void* fn = R == 1 ? (const void*)k_fcg<1> : (const void*)k_fcg<2>;
  cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(nb), dim3(FCG_TPB), args, 0, c->stream);
  c->launches++;
  if (e != cudaSuccess) return lv_cuda_check(c, e, "k_fcg cooperative launch");
  return LV_OK;
}
