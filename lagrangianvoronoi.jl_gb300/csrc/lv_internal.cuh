// Internal declarations shared by the CUDA translation units of liblvgpu.
//
// Device data layout (all FP64 unless noted, one entry per particle):
//   state   x, v, dv, momentum, Da (D11,D21), Db (D12,D22), GP : double2[cap]
//           e, P, rho, c2, mass, energy, quality, mu             : double[cap]
//           phase                                                : int32[cap]
//   mesh    per-polygon edge list and interior-face list in slot-major
//           ("ELL") layout: slot k of particle i lives at [k*cap + i], so a
//           warp reading slot k of 32 consecutive particles is coalesced.
//   cells   cell list as CSR over the n1*n2 cells: cstart[ncells+1],
//           citem[] (particle index), cpos[] (float2 offset of the copy from its
//           cell's lower corner; NaN for a periodic image).
//   solver  CSR of the pressure operator: rowptr[n+1], col[nnz], w[nnz]
//           (off-diagonal weights), adiag = diag + sum_j w_ij, dinv = 1/adiag.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/lvgpu.h"

#define LV_SIGNUM_EPS (2.0 * 2.220446049250313e-16) /* polygon.jl:2 */

// Layout of the device int array SolverDev::iters (per-solve statistics of
// one find_pressure call, slot = sweep index < 32, and solver flags).
#define LV_IT_ITERS 0          // [32] inner/CG iterations per slot
#define LV_IT_OUTER 32         // [32] refinement steps per slot
#define LV_IT_METHOD 64        // [32] method used per slot (learned solves)
#define LV_IT_JREF 128         // [32] iterations of the last Jacobi mixed solve per sweep slot
#define LV_IT_NONSINGULAR 97   // set when some diagonal term is nonzero
#define LV_IT_REDO 98          // polygons queued for the second clipping pass
#define LV_IT_FCG_BASE 100     // [2] arrivals and exchange epochs of the flag-reduced solver so far
#define LV_IT_SIZE 160

// Clock cycles a persistent solver waits on other blocks before it gives up
// and reports LV_ERR_BARRIER_TIMEOUT (about 2 s at 2 GHz; lv_set_wait_limit).
#define LV_WAIT_LIMIT_DEFAULT 4000000000LL

// Status bits set on the device with atomicOr; decoded on the host.
#define LV_FLAG_NAN_VELOCITY 0x1
#define LV_FLAG_MESH_DESTROYED 0x2
#define LV_FLAG_EDGE_OVERFLOW 0x4
#define LV_FLAG_CELL_OVERFLOW 0x8
#define LV_FLAG_NONFINITE 0x10
#define LV_FLAG_BARRIER_TIMEOUT 0x20
#define LV_FLAG_BAD_INPUT 0x40  // a field value the reference asserts against (heat_from_bdary!: cV > 0)

// Domain and cell-list constants passed to kernels by value.
struct GridDev {
  double bminx, bminy, bmaxx, bmaxy;  // boundary rectangle
  double cminx, cminy, cmaxx, cmaxy;  // cropping rectangle
  double ox, oy;                      // cell-list origin = cropping.xmin - (h, h)
  double h, rr_max, xperiod, yperiod, dr;
  double rh;                          // RN(1/h): the cell-key divisions by h through div_rcp
  double dx_hi, dy_hi;                // offsets from the origin beyond which a key is surely > n1 (> n2)
  int xper, yper;
  int n1, n2;
  int npath;
  float delta32;  // bound on the error of a candidate's float offset from the seed, per component
                  // (formed from the cell-relative offsets cpos and the path node's cell offset)
  float bigm;     // max |coordinate| inside the cropping box
  float h32;      // (float)h
  long long hxbits, hybits;  // bit patterns of 0.5 * xperiod, 0.5 * yperiod (get_arrow's wrap test)
  // a position whose float x lies strictly inside (ixlo, ixhi) has no
  // x-shifted periodic image in the cell grid (likewise y): the images only
  // reach the grid from within r_max + 2h of a periodic boundary
  float ixlo, ixhi, iylo, iyhi;
};

// One node of the candidate path (neighborlist.jl:29-41): cell offset and
// squared distance lower bound.
struct PathNodeDev {
  int di1, di2;
  double rr;
  float rrf;   // (float)rr, for the float test against the influence bound
  int beyond;  // rr > rr_max (only the last node of the clipping path)
};

struct StateDev {
  double2 *x, *v, *dv, *mom, *Da, *Db, *GP;
  double *e, *P, *rho, *c2, *mass, *energy, *quality, *mu;
  double *T, *kc, *cV;  // temperature, heat conductivity, specific heat (PolygonNSF, celldefs.jl:49-56)
  int* phase;
};

struct MeshDev {
  int cap;  // slot stride
  int* nedges;
  int* nfaces;
  double2 *ev1, *ev2;
  int* elab;
  int* fnbr;
  double *flrr, *flen;  // flen is filled on demand (lv_mesh_face_len)
  double2 *fm, *fy;
  double* area;
  double2* centroid;
  // The face kernels' thread -> row map: within each window of
  // LV_RPERM_WINDOW consecutive rows, the rows ordered by face count (stable),
  // so that the rows of a warp have nearly the same number of faces.  FP64
  // instructions are priced per warp on this GPU, and a warp runs its face
  // loop as often as its largest row needs.  Rebuilt by every remesh.
  int* rperm;
  // The clipping's polygon order: within each window of 1024 polygons,
  // ordered by the number of clips each needed in the previous
  // remesh (nclip; the particles move little between remeshes), so that
  // the polygons of a warp take about as many clip rounds each.
  unsigned char* nclip;
  int* cperm;
};
constexpr int LV_RPERM_WINDOW = 1024;  // (256: rhs 12.7, ops 11.8; 1024: 12.5, 11.5 ms per step at 4M)

// The row of face-kernel thread t (t < n).
__device__ __forceinline__ int face_row(const MeshDev& m, int t) { return __ldg(m.rperm + t); }

// RN(a / b) from y = RN(1/b) without a division (Markstein, IBM J. Res. Dev.
// 34(1), 1990): q0 = RN(a y) lies within 1.5 ulp of a/b, one correction
// q1 = RN(q0 + RN(a - b q0) y) within one ulp, and for such a q1 the residual
// a - b q1 is exact and RN(q1 + (a - b q1) y) is the correctly rounded
// quotient (Markstein's theorem).  For |a| outside [2^-900, 2^900) or |b|
// outside [2^-100, 2^100) (zeros, infinities, NaN, and every case where an
// intermediate could under- or overflow) the division itself.
__device__ __forceinline__ double div_rcp(double a, double b, double y) {
  const unsigned ea = ((unsigned)__double2hiint(a) >> 20) & 0x7ffu;
  const unsigned eb = ((unsigned)__double2hiint(b) >> 20) & 0x7ffu;
  if (ea - 123u < 1800u && eb - 923u < 200u) {
    double q = a * y;
    double r = fma(-b, q, a);
    q = fma(r, y, q);
    r = fma(-b, q, a);
    return fma(r, y, q);
  }
  return a / b;
}

// |v| > t for a double v and a positive finite t given by its bit pattern,
// on the integer pipe (the order of non-negative doubles is the order of
// their bit patterns; a NaN v compares greater, which the callers map to NaN
// either way).
__device__ __forceinline__ bool abs_greater(double v, long long tbits) {
  return (__double_as_longlong(v) & 0x7fffffffffffffffLL) > tbits;
}

// Epilogue of every pressure solve (one thread): the cumulative counters
// [0] solves, [1] iterations and [2] solves whose recursive (rr) or true (tr)
// residual is not within tol of ||b|| (NaN counts as not converged).
__device__ __forceinline__ void count_solve(long long* counters, int it, double rr, double bb, double tr,
                                            double tol2) {
  counters[0] += 1;
  counters[1] += it;
  if (!(rr <= tol2 * bb && tr <= tol2 * bb)) counters[2] += 1;
}

// The sweep's start P + c0 (P - pprev) + c1 D, rounded operation by
// operation (no contraction) so that every kernel that forms it agrees.
__device__ __forceinline__ double sweep_shift(double p, double pv, double d, double c0, double c1) {
  return __dadd_rn(__dadd_rn(p, __dmul_rn(c0, __dsub_rn(p, pv))), __dmul_rn(c1, d));
}

// Loads of data that no thread writes during the kernel, issued where they
// stand in the source (volatile inline PTX): the face and row loops load a
// batch of faces (entries) this way and only then use them, so that the
// loads are in flight together instead of one dependent round trip each.
__device__ __forceinline__ int ld_nc(const int* p) {
  int v;
  asm volatile("ld.global.nc.s32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ float ld_nc(const float* p) {
  float v;
  asm volatile("ld.global.nc.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ double ld_nc(const double* p) {
  double v;
  asm volatile("ld.global.nc.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ float4 ld_nc(const float4* p) {
  float4 v;
  asm volatile("ld.global.nc.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p));
  return v;
}
__device__ __forceinline__ double2 ld_nc(const double2* p) {
  double2 v;
  asm volatile("ld.global.nc.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "l"(p));
  return v;
}

// Face lengths |v1 - v2| of polygon i's interior edges in face order, with
// the expression of the reference's face loop.  The edges are loaded eight at
// a time (indexes clamped to the last edge) so that their loads overlap.
__device__ __forceinline__ void lv_face_lengths(const MeshDev& m, int i) {
  constexpr int B = 8;
  const int cap = m.cap, ne = m.nedges[i];
  int nf = 0;
  for (int k0 = 0; k0 < ne; k0 += B) {
    int lab[B];
    double2 a[B], b[B];
#pragma unroll
    for (int u = 0; u < B; ++u) {
      const size_t e = (size_t)min(k0 + u, ne - 1) * cap + i;
      lab[u] = ld_nc(m.elab + e);
      a[u] = ld_nc(m.ev1 + e);
      b[u] = ld_nc(m.ev2 + e);
    }
#pragma unroll
    for (int u = 0; u < B; ++u) {
      if (k0 + u < ne && lab[u] >= 0) {
        const double lx = a[u].x - b[u].x, ly = a[u].y - b[u].y;
        m.flen[(size_t)nf * cap + i] = sqrt(lx * lx + ly * ly);
        ++nf;
      }
    }
  }
}

struct CellsDev {
  int ncells;
  int* cstart;   // [ncells + 1]
  int* ccount;   // [ncells] counts
  int* citem;    // [item_cap]
  float2* cpos;  // [item_cap] offset from the cell's lower corner (NaN: a periodic image)
  int2* bkey;    // [images][cap]: cell and rank in the cell of every copy (re-binning)
  int item_cap;
};

struct SolverDev {
  int* rowptr;  // [cap + 1]
  int* col;     // [nnz_cap]
  double* w;    // [nnz_cap]
  float* w32;   // FP32 copy for the mixed-precision inner solve
  double *diag, *adiag, *dinv, *b, *xs, *r, *z, *p, *q, *tmp;
  // initial guess of find_pressure's sweeps (lv_sweep_sums): P and b before
  // the previous sweep's solve, d1 = P - pprev in FP32, block partials, the
  // coefficients c1, c2; dinc: the change of each sweep of the last call
  // (FP32, sweeps x cap, allocated with the first call that uses it)
  double *pprev, *bprev, *sgpart, *sgomega;
  float *sgd32, *dinc;
  int dinc_slots;
  float *dinv32, *r32, *z32, *p32, *q32, *d32, *e32, *f32a, *f32b;
  unsigned long long* rtag;  // staged solve: r of every row tagged with its exchange's epoch
  long long* counters; // [0] solves, [1] CG iterations, [2] solves that ended above the tolerance (cumulative)
  double* part;       // reduction partials [4][maxblocks]
  unsigned* bar;      // grid barrier {count, generation}
  int* iters;         // device-side stats
  double* dstats;     // device-side stats
  int64_t nnz_cap;
  unsigned long long* fslots;  // flag-published reduction words (lv_fcg.cu)
  // sweep-invariant RHS terms of refresh!, slot-major like the mesh faces
  double* rhs_tf;    // (lrr/dt) dot(v_i - v_j, m - y) per face
  double2* rhs_dmz;  // m - midpoint(x_i, y) per face
  double* rhs_te;    // dot(dS, vbc - v_i)/dt per boundary edge
  double2* rhs_dm;   // m - x_i per face
  double* rhs_den;   // rho c2 dt^2 per particle
  double* rhs_rden;  // RN(1 / rhs_den)
  double* rhs_rm;    // RN(1 / mass)
  // explicit learned M^-1 on the two-hop pattern (lv_fcg.cu, allocated on first use)
  int *mcnt = nullptr, *mcol = nullptr;
  float *mval = nullptr, *mdiag = nullptr;
  int* mok = nullptr;
  // the streaming solver's learned preconditioner in factored form (one-hop
  // pattern, systems beyond the staged solver): the same buffers hold G's
  // lower entries of each row in slots [0, nl), the entries G_ki (k > i) of
  // its column in slots [LV_MAX_EDGES, LV_MAX_EDGES + nu), mcnt = nl | nu << 8
  // and mdiag = G_ii, so M^-1 r = D^-1/2 (G^T G + eps I) D^-1/2 r is applied
  // as two one-hop passes instead of an explicit two-hop row
  bool mfac = false;
  int mrows = 0;
  // staged learned solve (lv_fcg.cu): per-block images, the operator's
  // columns remapped to shared-memory slots, build status [ok, max halo,
  // max ext, max entries]; whether the images of the current factor fit
  void* stage = nullptr;
  int *remap = nullptr, *stage_stat = nullptr;
  bool stage_ready = false;
  int stage_max[3] = {0, 0, 0};
  // streaming solver of large systems (lv_fcg.cu k_big, allocated on first
  // use): the operator's weights in the slot-major face layout (written by
  // the assembly while allocated), the FP32 vectors r u w p s d, the FP64
  // residual, the per-block neighbour masks and the synchronisation words
  float* ew32 = nullptr;
  double* ew64 = nullptr;
  float* bvec = nullptr;
  double* br64 = nullptr;
  unsigned* bmasks = nullptr;
  unsigned* bsync = nullptr;
  // MINRES (lv_fcg.cu k_minres, allocated on first use): r1, r2, w, w1, w2
  // and its synchronisation words
  double* mrvec = nullptr;
  unsigned* mrsync = nullptr;
};

struct LearnState;  // learned preconditioner (lv_learn.cu)

struct lv_ctx {
  lv_params prm;
  GridDev g;
  std::vector<PathNodeDev> path_host;
  PathNodeDev* path = nullptr;
  int dev = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  int n = 0;
  int cap = 0;
  bool meshed = false;
  StateDev s{};
  MeshDev m{};
  CellsDev c{};
  SolverDev sv{};
  int* status = nullptr;      // device status word
  int* status_host = nullptr; // pinned
  int method = LV_METHOD_MINRES;  // the reference's PressureSolver (pressure.jl:142-159, 219)
  double tol = 1e-6;
  int itmax = 1000;
  bool op_ready = false;
  double* mp_buf = nullptr;  // multiphase projection vectors (allocated on first use)
  LearnState* learn = nullptr;
  bool factor_valid = false;  // learned factor matches the assembled operator and parameters
  bool sweep_guess = true;  // Galerkin initial guess of the sweeps (LVGPU_SWEEP_GUESS=0 turns it off)
  // the sweep's start, queued by lv_solver_sweep_guess and applied by the next
  // solve of that vector: inside the flag-reduced solver, else by k_sweep_apply
  bool sg_pending = false;
  int sg_shift = 0;
  double* sg_P = nullptr;
  const float* sg_D = nullptr;
  float* sg_store = nullptr;
  int sg_valid = 0;         // sweeps of the last find_pressure whose changes sv.dinc holds
  int sg_n = 0;             // the particle count they belong to
  bool fcg_halo = true;    // staged mode of the learned one-block-per-SM solve (LVGPU_FCG_HALO=0 turns it off)
  bool fcg_reset = true;   // clear the flag-reduced solver's counter, flags and bases before its next launch
  long long spin_limit = LV_WAIT_LIMIT_DEFAULT;  // cycles a solver waits on other blocks (lv_set_wait_limit)
  int clip_slots = 0;      // first clipping pass's edge slots (0: the default; LVGPU_CLIP_SLOTS)
  bool big_reset = true;   // the same for the streaming solver's
  bool mr_reset = true;    // the same for MINRES's
  bool big_masks_valid = false;  // its neighbour masks match the operator
  bool big_masks_m = false;      // and cover M^-1's pattern
  bool flen_valid = false;  // m.flen belongs to the current mesh
  bool ccount_clean = false;  // the cell counts are zero (cleared by the last completed order pass)
  void* clip_resume = nullptr;  // captures of the first clipping pass (cap entries, allocated on first use)
  // boundary edges of the current mesh: per-polygon counts and offsets, the
  // count, room for per-edge values (velocity, charfun flag, label)
  int* bnd_cnt = nullptr;
  int* bnd_off = nullptr;
  int bnd_count = 0;
  int bnd_room = 0;
  bool bnd_valid = false;
  double2* bnd_vel = nullptr;
  unsigned char* bnd_act = nullptr;
  int* bnd_lab = nullptr;
  const double2* rhs_bvel = nullptr;  // per-edge boundary velocities of the running lv_find_pressure_edges
  // implicit viscous system (ViscousSolver): CSR of the face pattern, entries,
  // diagonal, right-hand side and iterate (2 cap interleaved unknowns)
  int* vs_rowptr = nullptr;
  int* vs_col = nullptr;
  double* vs_w = nullptr;
  double* vs_diag = nullptr;
  double* vs_b = nullptr;
  double* vs_u = nullptr;
  float learn_eps = 1e-4f;  // eps of M^-1 = D^-1/2 (Gt^T Gt + eps I) D^-1/2
  std::string err;
  int64_t launches = 0;
  // timings
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double t_ms[4] = {0, 0, 0, 0};
  bool timing = false;
  std::vector<void*> allocs;
  // per-family kernel timing (lv_kernel_timing)
  bool ktiming = false;
  struct KEvents {
    std::vector<cudaEvent_t> ev;  // start/end pairs
    size_t used = 0;              // events recorded since the last reset
    int64_t launches = 0;
  } kev[LV_KF_COUNT];
};

// Initial guess of find_pressure's sweep k: the solve of A P_k = b_k starts
// from P + c1 d1 + c2 D, the Galerkin projection of its error onto the span
// of two directions in the A-norm (exact minimisation of that error over the
// span; c = 0 is the plain warm start from P):
//   d1 = P - pprev, the last sweep's change (sweeps k >= 2);
//   D  = the change of sweep k in the previous call (sweeps the previous call
//        ran; the sweeps of consecutive time steps follow similar paths).
// The residual of the start is res = b_k - A P: for k >= 2 it equals
// (b_k - b_{k-1}) + the previous solve's residual, which the solver left
// below its tolerance and is dropped; for k = 1 (a new operator) it is
// evaluated.  For a singular operator res is taken projected to zero mean.
// (res, d1) and (res, D) are summed in FP64, the Gram entries (d, A d) in
// FP32 (only their relative size matters).  Called by every thread of the
// right-hand side's pass (blockDim.x == 256, `on` = row in range): block
// partials into sv.sgpart, the last block to finish adds them in block order
// and writes c1, c2 to sv.sgomega[0..1] (counter: zero before, zero after).
constexpr int LV_SG_TPB = 256;
constexpr int LV_SG_SUMS = 8;
__device__ __forceinline__ void lv_sweep_sums(const SolverDev& sv, int i, bool on, double res, double d1,
                                              const float* __restrict__ D, bool has1, bool has2, int n) {
  const bool singular = sv.iters[LV_IT_NONSINGULAR] == 0;
  // (res,d1) (res,D) (d1,Ad1) (d1,AD) (D,AD) sum res, sum d1, sum D
  double acc[LV_SG_SUMS] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (on) {
    const float f1 = has1 ? sv.sgd32[i] : 0.f;
    const float f2 = has2 ? D[i] : 0.f;
    const float dg = sv.d32[i];
    float a1 = dg * f1, a2 = dg * f2;
    const int e0 = sv.rowptr[i], e1 = sv.rowptr[i + 1];
    // entries eight at a time (indexes clamped to the row's last) so that
    // their loads overlap; the sums run over the entries in order
    constexpr int EB = 8;
    for (int b0 = e0; b0 < e1; b0 += EB) {
      int j[EB];
      float w[EB], g1[EB], g2[EB];
#pragma unroll
      for (int u = 0; u < EB; ++u) {
        const int e = min(b0 + u, e1 - 1);
        j[u] = ld_nc(sv.col + e);
        w[u] = ld_nc(sv.w32 + e);
      }
#pragma unroll
      for (int u = 0; u < EB; ++u) {
        g1[u] = has1 ? ld_nc(sv.sgd32 + j[u]) : 0.f;
        g2[u] = has2 ? ld_nc(D + j[u]) : 0.f;
      }
#pragma unroll
      for (int u = 0; u < EB; ++u) {
        if (b0 + u >= e1) break;
        if (has1) a1 = a1 + w[u] * (f1 - g1[u]);
        if (has2) a2 = a2 + w[u] * (f2 - g2[u]);
      }
    }
    acc[0] = res * d1;
    acc[1] = res * (double)f2;
    acc[2] = (double)(f1 * a1);
    acc[3] = (double)(f1 * a2);
    acc[4] = (double)(f2 * a2);
    acc[5] = res;
    acc[6] = d1;
    acc[7] = (double)f2;
  }
  // The block's sums: warp q adds sum q over the block's threads (eight
  // values per lane, then five shuffle levels).  FP64 additions are priced
  // per warp instruction on this GPU, so one warp per sum instead of a
  // shuffle tree in every warp.
  __shared__ double sh[LV_SG_SUMS][LV_SG_TPB];
  __shared__ bool s_last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nsum = singular ? LV_SG_SUMS : 5;
#pragma unroll
  for (int q = 0; q < LV_SG_SUMS; ++q)
    if (q < nsum) sh[q][threadIdx.x] = acc[q];
  __syncthreads();
  if (wid < nsum) {
    double v = 0.0;
#pragma unroll
    for (int k = 0; k < LV_SG_TPB / 32; ++k) v += sh[wid][lane + 32 * k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) {
      sv.sgpart[(size_t)wid * gridDim.x + blockIdx.x] = v;
      __threadfence();
    }
  }
  __syncthreads();
  unsigned* counter = sv.bar + 3;
  if (threadIdx.x == 0) s_last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // every block's partials of every sum, the loads of all sums together
  double pv[LV_SG_SUMS];
#pragma unroll
  for (int q = 0; q < LV_SG_SUMS; ++q) pv[q] = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += LV_SG_TPB) {
#pragma unroll
    for (int q = 0; q < LV_SG_SUMS; ++q)
      if (q < nsum) pv[q] += __ldcg(sv.sgpart + (size_t)q * gridDim.x + b);
  }
#pragma unroll
  for (int q = 0; q < LV_SG_SUMS; ++q) {
    if (q >= nsum) break;
    double v = pv[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) sh[q][wid] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t[LV_SG_SUMS] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int q = 0; q < LV_SG_SUMS; ++q)
      if (q < nsum)
        for (int k = 0; k < LV_SG_TPB / 32; ++k) t[q] += sh[q][k];
    double r1 = t[0], r2 = t[1];
    if (singular) {
      r1 -= t[5] * t[6] / (double)n;
      r2 -= t[5] * t[7] / (double)n;
    }
    const double a11 = t[2], a12 = t[3], a22 = t[4];
    double c1 = 0.0, c2 = 0.0;
    const bool u1 = has1 && a11 > 0.0, u2 = has2 && a22 > 0.0;
    const double det = a11 * a22 - a12 * a12;
    if (u1 && u2 && det > 1e-6 * a11 * a22) {  // else a nearly dependent pair
      c1 = (r1 * a22 - r2 * a12) / det;
      c2 = (a11 * r2 - a12 * r1) / det;
    } else if (u1 && (!u2 || r1 * r1 / a11 >= r2 * r2 / a22)) {
      c1 = r1 / a11;  // the better single direction (larger decrease of the error)
    } else if (u2) {
      c2 = r2 / a22;
    }
    if (!(c1 > -4.0 && c1 < 4.0 && c2 > -4.0 && c2 < 4.0)) c1 = c2 = 0.0;  // also NaN
    sv.sgomega[0] = c1;
    sv.sgomega[1] = c2;
    *counter = 0u;
  }
}

// Brackets the launches of one kernel family with CUDA events when kernel
// timing is on (lv_api.cu).
struct KernelTimer {
  lv_ctx* c;
  int fam;
  KernelTimer(lv_ctx* cc, int f);
  ~KernelTimer();
};

// ---- host helpers (lv_api.cu)
int lv_fail(lv_ctx* c, int code, const std::string& msg);
int lv_cuda_check(lv_ctx* c, cudaError_t e, const char* what);

// ---- mesh (lv_mesh.cu)
int lv_mesh_remesh(lv_ctx* c);
int lv_mesh_face_len(lv_ctx* c);  // fills m.flen unless it is current
int lv_mesh_captures_count(lv_ctx* c, int* count);  // second-pass polygons of the last remesh (synchronises)
int lv_scan_int(lv_ctx* c, const int* in, int* out, int len);  // exclusive, out[len] = total

// ---- per-device set-up (function attributes), once per device and process
#define LV_MAX_DEVICES 64
int lv_device_setup(int dev);  // lv_api.cu; call with dev current
int lv_mesh_device_setup();    // lv_mesh.cu
int lv_fcg_device_setup();     // lv_fcg.cu
int lv_learn_device_setup();   // lv_learn.cu

// ---- physics (lv_physics.cu)
int lv_phys_move(lv_ctx* c, double dt);
int lv_phys_eos(lv_ctx* c, int kind, double gamma, double p);
int lv_phys_gravity(lv_ctx* c, double gx, double gy, double dt);
int lv_phys_pressure_step(lv_ctx* c, double dt);
int lv_phys_find_D(lv_ctx* c);
int lv_phys_viscous(lv_ctx* c, double dt, int av);
// vwall: the label table (bvel null) or ignored; bvel/act: per boundary edge
// (lv_bnd_upload), act may be null
int lv_phys_friction(lv_ctx* c, const double* vwall, double dt, const double2* bvel = nullptr,
                     const unsigned char* act = nullptr);
// boundary edges of the current mesh (lv_physics.cu): offsets (once per mesh,
// synchronises), the list of midpoints and labels, per-edge values
int lv_bnd_prepare(lv_ctx* c);
int lv_bnd_list(lv_ctx* c, double* mid, int* lab);
int lv_bnd_upload(lv_ctx* c, int64_t nb, const double* vb, const unsigned char* act);
// Fourier heat conduction (fourier.jl) and the implicit viscous step (viscous_solver.jl)
int lv_phys_ideal_temperature(lv_ctx* c);
int lv_phys_fourier(lv_ctx* c, double dt);
int lv_phys_heat_bdary(lv_ctx* c, int64_t nb, const double* Tb, double dt);
int lv_phys_viscous_implicit(lv_ctx* c, double dt);
#define LV_VISC_SLOT 31  // stats slot of the implicit viscous solve
int lv_phys_find_dv(lv_ctx* c, double dt, double alpha);
int lv_phys_relax(lv_ctx* c, double dt, int rusanov);
// prepare = 1 evaluates the sweep-invariant terms (first sweep of find_pressure!)
// guess: also the sums of the sweep's initial guess (lv_sweep_sums) on the
// first (gp_step = 0) or the second pass; D: the previous call's change of this
// sweep (nullptr: none)
int lv_phys_rhs(lv_ctx* c, double dt, int gp_step, const double* vbc, int prepare, int guess = 0,
                const float* D = nullptr);
int lv_phys_multiphase(lv_ctx* c, double quality_threshold, lv_solve_stats* st);

// ---- learned preconditioner (lv_learn.cu)
int lv_learn_factor_current(lv_ctx* c);
void lv_learn_factor_ptrs(lv_ctx* c, const float** gd, const float** gl, const float** dh, const int** rev);
// two-hop part of the factor (all NULL with the one-hop pattern)
void lv_learn_factor2_ptrs(lv_ctx* c, const int** rowptr2, const int** col2, const float** gl2, const int** rev2);
void lv_learn_free(lv_ctx* c);

// ---- solver (lv_solver.cu)
int lv_solver_assemble(lv_ctx* c, double dt);
int lv_solver_solve(lv_ctx* c, double* dst_P, lv_solve_stats* st_dev_or_null, int stats_slot);
int lv_solver_apply(lv_ctx* c, const double* x_dev, double* y_dev);
// moves P to the sweep's start (c1, c2 from lv_sweep_sums), stores the last
// sweep's change into `store` (nullptr: none), saves P and b
int lv_solver_sweep_guess(lv_ctx* c, double* P, int it, const float* D, float* store);
int lv_solver_sweep_store(lv_ctx* c, const double* P, float* store);
int lv_solver_fetch_stats(lv_ctx* c, lv_solve_stats* out, int count);

// ---- flag-reduced mixed-precision solver (lv_fcg.cu)
#define LV_FCG_SLOT_WORDS (8192 + 16 * 1024)  // u64: partial words, then 128-byte exchange flags
int lv_fcg_capacity(lv_ctx* c);
int lv_fcg_build_minv(lv_ctx* c);
int lv_fcg_solve(lv_ctx* c, double* x, int slot, bool learned);
int lv_solver_flush_shift(lv_ctx* c);  // applies a queued sweep start (k_sweep_apply)
int lv_fcg_halo_info(lv_ctx* c, int* max_rows);
void lv_fcg_free(lv_ctx* c);
// streaming solver of systems above lv_fcg_capacity (same methods)
int lv_big_prepare(lv_ctx* c);  // allocations; called before the assembly of such a system
int lv_big_solve(lv_ctx* c, double* x, int slot, bool learned);
// MINRES without a preconditioner (LV_METHOD_MINRES), any size
int lv_minres_solve(lv_ctx* c, double* x, int slot);
// the same kernel on another operator: ncomp unknowns per particle
// (interleaved), eform 1 the ThreadedMat row form (entries, then the diagonal)
int lv_minres_general(lv_ctx* c, const int* rowptr, const int* col, const double* w, const double* diag,
                      const double* b, double* x, int ncomp, int eform, double tol, int itmax, int slot);

#define LV_LAUNCH_CHECK(c, what)                                   \
  do {                                                             \
    (c)->launches++;                                               \
    cudaError_t _e = cudaGetLastError();                           \
    if (_e != cudaSuccess) return lv_cuda_check((c), _e, (what));  \
  } while (0)

static inline int lv_blocks(int n, int tpb) { return (n + tpb - 1) / tpb; }
