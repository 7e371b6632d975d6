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
#include <algorithm>
#include <cstddef>
#include <cstdlib>
#include <mutex>

#include "lv_internal.cuh"

namespace {

constexpr int FCG_TPB = 512;
constexpr int FKR = 8;    // operator entries per row held in registers
constexpr int FKM = 12;   // preconditioner off-diagonal entries per row held in registers
constexpr int MMAX = 96;  // preconditioner off-diagonal entries per row (storage slots)
constexpr long long FCG_SPIN_LIMIT = LV_WAIT_LIMIT_DEFAULT;  // cycles: the bulk copies' waits
constexpr float FCG_UPDATE_DROP = 1e-5f;  // FP32 residual reduction per refinement step
constexpr int FCG_MAX_UPDATES = 200;

constexpr int RG_WORDS = 4;  // partial-sum words per block and phase
constexpr int FCG_RPB_MAX = FCG_TPB * 2;  // rows per block at most (two per thread)
constexpr int FCG_HMAX = 1536;            // staged mode: halo rows per block
constexpr int STG_EXTMAX = 2048;          // staged mode: r values a block gathers per iteration
constexpr int STG_MAXG = FCG_RPB_MAX / 32 + FCG_HMAX / 32;  // row groups of 32
constexpr int STG_PMAX = FCG_RPB_MAX + FCG_HMAX;  // staged mode: rows whose u a block computes
constexpr int STG_ENTRIES = 24576;  // staged mode: M^-1 entries per block (padded per group)
constexpr int STG_SLOTS = 32;       // staged mode: M^-1 off-diagonal entries per row at most
constexpr int STG_HASH = 8192;      // hash slots of the image builder
constexpr int FLAG_STRIDE = 32;  // exchange flags sit on separate 128-byte lines (packed flags halve the speed)
constexpr int FCG_MAX_BLOCKS = 1024;

// Tagged values: the high word is the exchange's epoch with the top bit set
// (zeroed memory never matches), the low word the float's bits.  An aligned
// 64-bit access is single-copy atomic, so a word whose tag is current also
// holds the current value: no flag and no fence are needed.
__device__ __forceinline__ unsigned rtag_of(unsigned ee) { return ee | 0x80000000u; }
__device__ __forceinline__ void st_tagged(unsigned long long* p, unsigned tag, float v) {
  const unsigned long long w = ((unsigned long long)tag << 32) | __float_as_uint(v);
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(w) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Per-block image of the staged learned solve, built once per factor by
// k_stage_build and moved to shared memory at launch (bulk copies of each
// field's used prefix, below).  The rows whose u the
// block computes (its own rows and its halo: the rows outside the block that
// its operator rows reference) take positions ordered by their M^-1 entry
// count, longest first; thread t applies positions t, t + 512, ...  Positions
// form groups of 32, stored slot-major within a group and padded to the
// group's longest row (one warp reads one slot of 32 rows without bank
// conflicts; the ordering keeps the padding small).  Column indices point into
// the block's r staging: own rows first, then the ext rows gathered from
// other blocks.
struct StageImage {
  int npos, ne, nh, total;  // positions, ext rows, halo rows, entries
  int goff[STG_MAXG];       // first entry of each group
  int gsl[STG_MAXG];        // slots of each group
  int ext[STG_EXTMAX];      // rows gathered from other blocks each iteration
  float pmd[STG_PMAX];      // per position: M^-1 diagonal
  float pdnv[STG_PMAX];     // per position: Jacobi scale
  unsigned short pridx[STG_PMAX];  // per position: the row's r in the staging
  unsigned short puidx[STG_PMAX];  // per position: the row's u in shared memory
  unsigned char pm[STG_PMAX];      // per position: off-diagonal entries
  int hrow[FCG_HMAX];              // halo rows (global) by halo slot, for the FP64 residual
  float sval[STG_ENTRIES];
  unsigned short sidx[STG_ENTRIES];
};
static_assert(offsetof(StageImage, ext) % 16 == 0 && offsetof(StageImage, pmd) % 16 == 0 &&
                  offsetof(StageImage, pdnv) % 16 == 0 && offsetof(StageImage, pridx) % 16 == 0 &&
                  offsetof(StageImage, puidx) % 16 == 0 && offsetof(StageImage, pm) % 16 == 0 &&
                  offsetof(StageImage, hrow) % 16 == 0 && offsetof(StageImage, sval) % 16 == 0 &&
                  offsetof(StageImage, sidx) % 16 == 0 && sizeof(StageImage) % 16 == 0,
              "16-byte bulk copies of every field");

// Shared memory of the staged mode: r of the own rows then of the ext rows,
// u of the own rows then of the halo rows, the image.
struct StageSmem {
  float r[FCG_RPB_MAX + STG_EXTMAX];
  float u[FCG_RPB_MAX + FCG_HMAX];
  StageImage img;
};
static_assert(offsetof(StageSmem, img) % 16 == 0, "16-byte copies");

struct FcgArgs {
  int n, nb, rows_per_block;
  const int* rowptr;
  const int* col;
  const double* w;
  const float* w32;    // FP32 copies of w, diag, dinv (made when the operator is assembled)
  const float* dg32;
  const float* dinv32;
  const double* diag;  // the reference's diagonal term (mass part)
  const double* dinv;  // 1 / (diag + sum_j w_ij)
  const double* b;
  double* x;  // FP64 iterate, also the exchange buffer of the outer residual
  float* rbuf;
  float* ubuf;    // u exchange
  unsigned long long* rtag;  // staged mode: the r exchange as tagged words
  unsigned long long* slots;  // partial words [2 parities][RG_WORDS][nb] (as 32-bit words)
  unsigned* counter;          // arrivals, cumulative over launches
  unsigned* sync_base;        // [0] arrivals, [1] exchange epochs of the previous launches
  unsigned* flags;            // per-block exchange epochs, one 128-byte line each (FLAG_STRIDE words)
  int* status;
  double tol2;
  int itmax;
  long long spin;   // cycles a wait on another block lasts before it gives up
  const int* nonsingular;
  int learned;
  const int* mcnt;  // learned M^-1: off-diagonal count, slot-major entries, diagonal
  const int* mcol;
  const float* mval;
  const float* mdiag;
  int mstride;
  const int* minv_ok;
  // staged mode (learned): each block also computes u = M^-1 r on its halo,
  // so that only r crosses blocks; the operator's columns are remapped to
  // the shared-memory u of the own and halo rows
  const StageImage* stage;
  const int* remap;
  // the sweep's start, queued by the sweep guess (0: none; 1: keep P and b
  // for the next sweep; 2: also start from P + c0 (P - pprev) + c1 D)
  int sg_mode;
  double* pprev;
  double* bprev;
  const float* sgD;
  float* sgstore;
  const double* sgcoef;
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

// The arrival counter and the exchange flags are never reset: a launch
// continues from the totals the previous one left in sync_base (read into
// this block's shared s_base at the start), and comparisons are wrap-safe.
__shared__ unsigned s_base[2];

// thread 0: arrive and wait for phase ph; returns 0 on timeout
template <class Args>
__device__ __forceinline__ int arrive_wait(const Args& a, unsigned ph) {
  red_release_add(a.counter, 1u);
  const unsigned target = s_base[0] + ph * (unsigned)a.nb;
  const long long t0 = clock64();
  while ((int)(ld_acquire_u32(a.counter) - target) < 0) {
    if (clock64() - t0 > a.spin) {
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

template <int NV, typename T, class Args>
__device__ bool fphase(const Args& a, unsigned ph, const T (&v)[NV], T (&tot)[NV]) {
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
    for (int k = 0; k < NV; ++k)
      Words<T>::put(allsum(lane < (int)(blockDim.x >> 5) ? shw[k * 32 + lane] : T(0)), wd + k * Words<T>::N);
    if (lane == 0) {
#pragma unroll
      for (int q = 0; q < NWD; ++q) __stcg(words + (size_t)q * a.nb + blockIdx.x, wd[q]);
      s_ok = arrive_wait(a, ph);
    }
  }
  __syncthreads();
  if (!s_ok) return false;
  // 2. every block's words, read once: thread t reads block t's; only the
  // warps that hold words add (the FP64 pipe of this GPU is narrow), and one
  // thread forms the totals for the whole block
  __shared__ T s_tot[NV];
  const int nwr = (a.nb + 31) >> 5;  // warps holding words
  if (wid < nwr) {
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
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      T t = T(0);
      for (int q = 0; q < nwr; ++q) t += shw2[k * 32 + q];
      s_tot[k] = t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) tot[k] = s_tot[k];
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
template <class Args>
__device__ bool nexchange(const Args& a, unsigned e, const unsigned* mask) {
  __syncthreads();
  const unsigned ee = s_base[1] + e;
  if (threadIdx.x == 0) st_release_u32(a.flags + (size_t)blockIdx.x * FLAG_STRIDE, ee);
  int to = 0;
  const int t = threadIdx.x;
  if (t < a.nb && ((mask[t >> 5] >> (t & 31)) & 1u)) {
    const long long t0 = clock64();
    while ((int)(ld_acquire_u32(a.flags + (size_t)t * FLAG_STRIDE) - ee) < 0) {
      if (clock64() - t0 > a.spin) {
        to = 1;
        atomicOr(a.status, LV_FLAG_BARRIER_TIMEOUT);
        break;
      }
    }
  }
  return __syncthreads_or(to) == 0;
}

// The staged image is moved into shared memory by the bulk-copy engine
// (cp.async.bulk, no tensor map: 16-byte aligned addresses, sizes multiples
// of 16), completing on an mbarrier, while the threads load their rows and
// evaluate the first FP64 residual.
constexpr unsigned BULK_CHUNK = 16384;
__device__ __forceinline__ void mbar_init(unsigned long long* bar) {
  const unsigned b = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  const unsigned b = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(unsigned long long* bar, unsigned parity) {
  const unsigned b = (unsigned)__cvta_generic_to_shared(bar);
  unsigned done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(done)
      : "r"(b), "r"(parity)
      : "memory");
  return done != 0;
}
// bytes (a multiple of 16) from src to dst in chunks, completing on bar
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  const unsigned b = (unsigned)__cvta_generic_to_shared(bar);
  unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  const char* sp = static_cast<const char*>(src);
  for (unsigned off = 0; off < bytes; off += BULK_CHUNK) {
    const unsigned sz = min(BULK_CHUNK, bytes - off);
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     d + off),
                 "l"(sp + off), "r"(sz), "r"(b)
                 : "memory");
  }
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

// HALO: the staged instantiation (learned solves whose image fits shared
// memory); the other one is free of its code and holds M^-1 in registers.
template <int R, bool HALO>
__global__ void __launch_bounds__(FCG_TPB, 1) k_fcg(FcgArgs a) {
  const int n = a.n;
  const int rb0 = blockIdx.x * a.rows_per_block;
  const int rb1 = min(n, rb0 + a.rows_per_block);
  const bool learned0 = a.learned != 0 && *a.minv_ok != 0;
  if (threadIdx.x == 0) {
    s_base[0] = __ldcg(a.sync_base);
    s_base[1] = __ldcg(a.sync_base + 1);
  }  // visible after the first __syncthreads, before any phase or exchange
  extern __shared__ __align__(16) unsigned char fcg_dyn[];
  StageSmem& ss = *reinterpret_cast<StageSmem*>(fcg_dyn);
  // staged mode: the block's image in global memory; its copy in shared memory
  // is ready once img_ready is set (until then ext and the halo rows are read
  // from the global image)
  const StageImage* gim = HALO ? a.stage + blockIdx.x : nullptr;
  __shared__ __align__(8) unsigned long long s_img_bar;
  bool img_ready = !HALO;
  if constexpr (HALO) {
    if (threadIdx.x == 0) {
      // the used prefix of every field (each field starts on a 16-byte
      // boundary; sizes rounded up to 16 bytes stay inside the field)
      const int4 hd = *reinterpret_cast<const int4*>(gim);  // npos, ne, nh, total
      const unsigned npos = (unsigned)hd.x, ne = (unsigned)hd.y, nh = (unsigned)hd.z, total = (unsigned)hd.w;
      auto up16 = [](unsigned b) { return (b + 15u) & ~15u; };
      const unsigned hdr = (unsigned)offsetof(StageImage, ext);
      const unsigned sz[9] = {hdr,           up16(ne * 4u),   up16(npos * 4u), up16(npos * 4u), up16(npos * 2u),
                              up16(npos * 2u), up16(npos),   up16(nh * 4u),   total * 4u};
      const size_t off[9] = {0,
                             offsetof(StageImage, ext),
                             offsetof(StageImage, pmd),
                             offsetof(StageImage, pdnv),
                             offsetof(StageImage, pridx),
                             offsetof(StageImage, puidx),
                             offsetof(StageImage, pm),
                             offsetof(StageImage, hrow),
                             offsetof(StageImage, sval)};
      unsigned bytes = total * 2u;
      for (int f = 0; f < 9; ++f) bytes += sz[f];
      mbar_init(&s_img_bar);
      mbar_expect_tx(&s_img_bar, bytes);
      const char* src = reinterpret_cast<const char*>(gim);
      char* dst = reinterpret_cast<char*>(&ss.img);
      for (int f = 0; f < 9; ++f)
        if (sz[f]) bulk_g2s(dst + off[f], src + off[f], sz[f], &s_img_bar);
      if (total) bulk_g2s(ss.img.sidx, gim->sidx, total * 2u, &s_img_bar);
    }
  }
  // every thread waits for the image (bounded; on a timeout the copies get a
  // second bounded wait before the block may exit); the block agrees on the result
  auto img_wait = [&]() -> bool {
    bool fail = false;
    const long long t0 = clock64();
    while (!mbar_try(&s_img_bar, 0u)) {
      if (clock64() - t0 > FCG_SPIN_LIMIT) {
        fail = true;
        atomicOr(a.status, LV_FLAG_BARRIER_TIMEOUT);
        const long long t1 = clock64();
        while (!mbar_try(&s_img_bar, 0u) && clock64() - t1 < FCG_SPIN_LIMIT) {
        }
        break;
      }
    }
    return __syncthreads_or(fail) == 0;
  };
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
      rr.cc[k][e] = have ? (HALO ? a.remap[rr.beg[k] + e] : a.col[rr.beg[k] + e]) : 0;
      rr.ww[k][e] = have ? a.w32[rr.beg[k] + e] : 0.f;
    }
    rr.dg[k] = on ? a.dg32[i] : 0.f;
    rr.dnv[k] = on ? a.dinv32[i] : 0.f;
    rr.mn[k] = (on && learned0) ? a.mcnt[i] : 0;
    if constexpr (!HALO) {
#pragma unroll
      for (int e = 0; e < FKM; ++e) {
        const bool have = e < rr.mn[k];
        rr.mc[k][e] = have ? a.mcol[(size_t)e * a.mstride + i] : 0;
        rr.mv[k][e] = have ? a.mval[(size_t)e * a.mstride + i] : 0.f;
      }
    }
    rr.md[k] = (on && learned0) ? a.mdiag[i] : 0.f;
    rr.bb[k] = on ? a.b[i] : 0.0;
    x[k] = on ? a.x[i] : 0.0;
  }
  // the sweep's start: the own rows shift now; the halo rows are shifted
  // where the first residual gathers them; P (unshifted) goes to pprev and the
  // shifted x to P once every block has gathered (after the first phase)
  double pold[R];
  const double sgc0 = a.sg_mode == 2 ? a.sgcoef[0] : 0.0, sgc1 = a.sg_mode == 2 ? a.sgcoef[1] : 0.0;
#pragma unroll
  for (int k = 0; k < R; ++k) {
    pold[k] = x[k];
    if (a.sg_mode && rr.on[k]) {
      const int i = rr.i[k];
      const double pv = a.pprev[i];
      if (a.sgstore) a.sgstore[i] = (float)(x[k] - pv);
      if (a.sg_mode == 2) x[k] = sweep_shift(x[k], pv, a.sgD ? (double)a.sgD[i] : 0.0, sgc0, sgc1);
      a.bprev[i] = a.b[i];
    }
  }
  bool first_res = true;
  // x of row j as the first residual sees it (shifted when the start is)
  auto x_at = [&](int j) -> double {
    const double p = __ldcg(a.x + j);
    if (!first_res || a.sg_mode != 2) return p;
    return sweep_shift(p, __ldcg(a.pprev + j), a.sgD ? (double)__ldcg(a.sgD + j) : 0.0, sgc0, sgc1);
  };
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
    if constexpr (!HALO) {
#pragma unroll
      for (int k = 0; k < R; ++k) {
        if (!rr.on[k]) continue;
        for (int e = rr.beg[k]; e < rr.beg[k] + rr.cnt[k]; ++e) mark(a.col[e]);
        for (int e = 0; e < rr.mn[k]; ++e) mark(a.mcol[(size_t)e * a.mstride + rr.i[k]]);
      }
    }
    // staged mode: the owners of the gathered rows (these include every
    // operator column outside the block, i.e. the halo rows, and the columns
    // of every staged M^-1 row)
    if constexpr (HALO) {
      const int ne = gim->ne;
      for (int q = threadIdx.x; q < ne; q += FCG_TPB) mark(gim->ext[q]);
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
    __shared__ double s_mean;
    if (threadIdx.x == 0) s_mean = t[0] / (double)n;  // one FP64 division per block
    __syncthreads();
    const double mean = s_mean;
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
  // out = A v with the neighbours' values from buf (FP32 difference form);
  // in the staged mode from shared memory through the remapped columns
  auto spmv = [&](const float* buf, const float(&own)[R], float(&out)[R]) {
#pragma unroll
    for (int k = 0; k < R; ++k) {
      float acc = rr.dg[k] * own[k];
#pragma unroll
      for (int e = 0; e < FKR; ++e)
        if (e < rr.cnt[k]) {
          const float vj = HALO ? ss.u[rr.cc[k][e]] : __ldcg(buf + rr.cc[k][e]);
          acc = fmaf(rr.ww[k][e], own[k] - vj, acc);
        }
      for (int e = FKR; e < rr.cnt[k]; ++e) {
        const int q = rr.beg[k] + e;
        const float vj = HALO ? ss.u[a.remap[q]] : __ldcg(buf + a.col[q]);
        acc = fmaf(a.w32[q], own[k] - vj, acc);
      }
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
    if constexpr (HALO) {
      // r crosses blocks (global and staged); u of the own and the halo rows
      // lands in shared memory, each halo row computed exactly as its owner
      // computes it (same entries, same order)
      if (!img_ready) {
        if (!img_wait()) return false;
        img_ready = true;
      }
      const int rpb = a.rows_per_block;
      const int lane = threadIdx.x & 31;
      // the exchange: every row's r as a word tagged with this exchange's
      // epoch; a reader takes an ext row's word once its tag is current
      // (bounded), so it waits on the data itself, not on a flag and then
      // the data.  Consecutive exchanges are separated by a grid-wide phase,
      // so no word is overwritten before every reader has taken it.
      const unsigned tag = rtag_of(s_base[1] + (++xe));
#pragma unroll
      for (int k = 0; k < R; ++k)
        if (rr.on[k]) {
          st_tagged(a.rtag + rr.i[k], tag, r[k]);
          ss.r[threadIdx.x + k * FCG_TPB] = r[k];
        }
      const int ne = ss.img.ne;
      constexpr int NQ = STG_EXTMAX / FCG_TPB;
      float ev[NQ];
      unsigned long long wv[NQ];
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const int e = threadIdx.x + q * FCG_TPB;
        wv[q] = e < ne ? ld_relaxed_u64(a.rtag + ss.img.ext[e]) : ((unsigned long long)tag << 32);
      }
      int late = 0;
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const int e = threadIdx.x + q * FCG_TPB;
        if ((unsigned)(wv[q] >> 32) != tag) {
          const long long t0 = clock64();
          do {
            wv[q] = ld_relaxed_u64(a.rtag + ss.img.ext[e]);
            if (clock64() - t0 > a.spin) {
              late = 1;
              atomicOr(a.status, LV_FLAG_BARRIER_TIMEOUT);
              break;
            }
          } while ((unsigned)(wv[q] >> 32) != tag);
        }
        ev[q] = __uint_as_float((unsigned)wv[q]);
      }
      if (__syncthreads_or(late)) return false;
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const int e = threadIdx.x + q * FCG_TPB;
        if (e < ne) ss.r[rpb + e] = ev[q];
      }
      __syncthreads();
      // u at this thread's positions p = t + k 512: u_i = md_i r_i + the
      // row's slots in order (a halo row exactly as its owner computes it),
      // or the Jacobi scale times r_i.  The loads of four
      // slots are issued together (padding slots point at a valid index with
      // value 0 and are not added).
      auto row_apply = [&](int g, int m, float md, float ri) {
        const int base = ss.img.goff[g] + lane;
        const int sl = ss.img.gsl[g];
        float t = md * ri;
        int q = 0;
        for (; q + 4 <= sl; q += 4) {
          float v[4], xr[4];
#pragma unroll
          for (int z = 0; z < 4; ++z) {
            v[z] = ss.img.sval[base + (q + z) * 32];
            xr[z] = ss.r[ss.img.sidx[base + (q + z) * 32]];
          }
#pragma unroll
          for (int z = 0; z < 4; ++z)
            if (q + z < m) t = fmaf(v[z], xr[z], t);
        }
        for (; q < sl; ++q)
          if (q < m) t = fmaf(ss.img.sval[base + q * 32], ss.r[ss.img.sidx[base + q * 32]], t);
        return t;
      };
      constexpr int KP = STG_PMAX / FCG_TPB;
      const int npos = ss.img.npos;
      float acc[KP];
#pragma unroll
      for (int k = 0; k < KP; ++k) {
        const int p = threadIdx.x + k * FCG_TPB;
        acc[k] = 0.f;
        if (p < npos) {
          const float ri = ss.r[ss.img.pridx[p]];
          acc[k] = learned ? row_apply(p >> 5, ss.img.pm[p], ss.img.pmd[p], ri) : ss.img.pdnv[p] * ri;
        }
      }
#pragma unroll
      for (int k = 0; k < KP; ++k) {
        const int p = threadIdx.x + k * FCG_TPB;
        if (p < npos) ss.u[ss.img.puidx[p]] = acc[k];
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < R; ++k) u[k] = rr.on[k] ? ss.u[threadIdx.x + k * FCG_TPB] : 0.f;  // zeros past the block's end
    } else {
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
    if constexpr (HALO) {
      // x of the own rows and of the halo in shared memory (the float
      // staging is free between iterations), gathered like u
      double* xo = reinterpret_cast<double*>(ss.u);
      double* xh = reinterpret_cast<double*>(ss.r);
      static_assert(sizeof(ss.u) >= sizeof(double) * FCG_RPB_MAX && sizeof(ss.r) >= sizeof(double) * FCG_HMAX,
                    "FP64 staging fits the float staging");
#pragma unroll
      for (int k = 0; k < R; ++k)
        if (rr.on[k]) xo[threadIdx.x + k * FCG_TPB] = x[k];
      const StageImage* im = img_ready ? &ss.img : gim;  // the halo rows, staged or global
      const int nh = im->nh;
      double xv[FCG_HMAX / FCG_TPB];
#pragma unroll
      for (int q = 0; q < FCG_HMAX / FCG_TPB; ++q) {
        const int h = threadIdx.x + q * FCG_TPB;
        xv[q] = h < nh ? x_at(im->hrow[h]) : 0.0;
      }
#pragma unroll
      for (int q = 0; q < FCG_HMAX / FCG_TPB; ++q) {
        const int h = threadIdx.x + q * FCG_TPB;
        if (h < nh) xh[h] = xv[q];
      }
      __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
      double acc = 0.0;
      if (rr.on[k]) {
        acc = a.diag[rr.i[k]] * x[k];
        if constexpr (HALO) {
          // columns remapped to own rows (< rows_per_block) and halo slots
          const double* xo = reinterpret_cast<const double*>(ss.u);
          const double* xh = reinterpret_cast<const double*>(ss.r);
          const int rpb = a.rows_per_block;
#pragma unroll
          for (int e = 0; e < FKR; ++e)
            if (e < rr.cnt[k]) {
              const int cc = rr.cc[k][e];
              acc += a.w[rr.beg[k] + e] * (x[k] - (cc < rpb ? xo[cc] : xh[cc - rpb]));
            }
          for (int e = FKR; e < rr.cnt[k]; ++e) {
            const int cc = a.remap[rr.beg[k] + e];
            acc += a.w[rr.beg[k] + e] * (x[k] - (cc < rpb ? xo[cc] : xh[cc - rpb]));
          }
        } else {
          for (int e = rr.beg[k]; e < rr.beg[k] + rr.cnt[k]; ++e) acc += a.w[e] * (x[k] - x_at(a.col[e]));
        }
      }
      r64[k] = rr.on[k] ? rr.bb[k] - acc : 0.0;
      v[0] += r64[k] * r64[k];
      v[1] += rr.bb[k] * rr.bb[k];
    }
    if (!(ok = fphase<2, double>(a, ++ep, v, t2))) break;
    if (first_res) {
      // every block has gathered its halo of the unshifted P
      first_res = false;
      if (a.sg_mode) {
#pragma unroll
        for (int k = 0; k < R; ++k)
          if (rr.on[k]) {
            a.pprev[rr.i[k]] = pold[k];
            if (a.sg_mode == 2) a.x[rr.i[k]] = x[k];
          }
      }
    }
    rtrue2 = t2[0];
    bnorm2 = t2[1];
    if (rtrue2 <= a.tol2 * bnorm2 || it >= a.itmax || updates >= FCG_MAX_UPDATES) break;
    // the restart's scalars once per block (the FP64 square root and
    // divisions are many FP64 instructions on this GPU)
    __shared__ double s_sig[2];
    __shared__ float s_rho_upd;
    if (threadIdx.x == 0) {
      const double sg = sqrt(rtrue2);
      s_sig[0] = sg;
      s_sig[1] = 1.0 / sg;
      s_rho_upd = fmaxf(FCG_UPDATE_DROP * FCG_UPDATE_DROP, (float)(0.25 * a.tol2 * bnorm2 / rtrue2));
    }
    __syncthreads();
    sigma = s_sig[0];
    const double inv_sigma = s_sig[1];
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
    const float rho_upd = s_rho_upd;
    if (!(ok = precond())) break;
    while (true) {
      if constexpr (!HALO) {
#pragma unroll
        for (int k = 0; k < R; ++k)
          if (rr.on[k]) a.ubuf[rr.i[k]] = u[k];
        if (!(ok = nexchange(a, ++xe, s_mask))) break;
      }
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
  // no bulk copy may still be in flight when the block exits
  if (!img_ready) img_wait();
  if (ok && blockIdx.x == 0 && threadIdx.x == 0) {
    // every block read the bases before its first arrival, and this is after
    // the last phase: the next launch continues from here
    a.sync_base[0] = s_base[0] + ep * (unsigned)a.nb;
    a.sync_base[1] = s_base[1] + xe;
    *a.out_iters = it;
    *a.out_outer = updates;
    *a.out_method = learned ? LV_METHOD_LEARNED_PCG : LV_METHOD_MIXED_IR;
    if (!a.learned) *a.jref = it;
    a.out_d[0] = rtrue2;
    a.out_d[1] = bnorm2;
    a.out_d[2] = rtrue2;
    count_solve(a.counters, it, rtrue2, bnorm2, rtrue2, a.tol2);
  }
}

// M^-1 = D^-1/2 (Gt^T Gt + eps I) D^-1/2, one thread per row i:
// (Gt^T Gt)_ij = sum_k Gt_ki Gt_kj over k in {i} and the rows whose pattern
// holds i (the upper neighbours of i, and with the two-hop pattern its upper
// two-hop neighbours), j over the pattern of row k (k, its lower neighbours
// and lower two-hop neighbours).  Two hops of Gt give M^-1 two (one-hop
// pattern) or four (two-hop pattern) hops.
// only: rows whose flag is set (nullptr: every row)
__global__ void k_build_minv(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                             const float* __restrict__ gd, const float* __restrict__ gl, const int* __restrict__ rev,
                             const int* __restrict__ rowptr2, const int* __restrict__ col2,
                             const float* __restrict__ gl2, const int* __restrict__ rev2,
                             const float* __restrict__ dh, float eps, int stride, int* mcnt, int* mcol, float* mval,
                             float* mdiag, int* ok, const int* __restrict__ only) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (only && !only[i]) return;
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

// The staged image of solve block b (rows [b rpb, (b+1) rpb)), one block of
// STG_BUILD_TPB threads per solve block.  An open-addressing hash in shared
// memory numbers the rows outside the block: first the halo (the operator's
// columns), then the rest of the ext rows (the M^-1 columns of the own and the
// halo rows).  Then it writes the image and remaps every operator nonzero of
// the block's rows to the shared-memory u of the staged solve (own row j:
// j - b rpb; halo row: rpb + halo slot).  stat[0] is cleared when an image
// does not fit; stat[1..3] collect the largest halo, ext and entry counts.
constexpr int STG_BUILD_TPB = 1024;
constexpr size_t STG_BUILD_SMEM = (size_t)STG_HASH * (4 + 2 + 2) + (size_t)FCG_HMAX * 4 + (size_t)STG_PMAX * 4;

__device__ __forceinline__ unsigned stg_hash(int j) { return ((unsigned)j * 2654435761u) >> 19; }

__global__ void __launch_bounds__(STG_BUILD_TPB) k_stage_build(int n, int rpb, const int* __restrict__ rowptr,
                                                               const int* __restrict__ col,
                                                               const int* __restrict__ mcnt,
                                                               const int* __restrict__ mcol,
                                                               const float* __restrict__ mval,
                                                               const float* __restrict__ mdiag,
                                                               const double* __restrict__ dinv, int mstride,
                                                               StageImage* images, int* remap, int* stat) {
  static_assert(STG_HASH == 8192, "stg_hash yields 13 bits");
  extern __shared__ __align__(16) unsigned char stg_dyn[];
  int* keys = reinterpret_cast<int*>(stg_dyn);
  short* hsl = reinterpret_cast<short*>(keys + STG_HASH);
  short* esl = hsl + STG_HASH;
  int* hrow = reinterpret_cast<int*>(esl + STG_HASH);
  int* prow = hrow + FCG_HMAX;  // sorted position -> unsorted (own rows, then halo rows)
  __shared__ int s_nh, s_ne, s_bad, s_total;
  __shared__ int s_gsl[STG_MAXG], s_goff[STG_MAXG];
  __shared__ int s_hist[STG_SLOTS + 1];
  const int b = blockIdx.x, t = threadIdx.x;
  const int lane = t & 31, wid = t >> 5;
  StageImage& im = images[b];
  const int rb0 = b * rpb, rb1 = min(n, rb0 + rpb);
  const int nown = max(0, rb1 - rb0);
  for (int h = t; h < STG_HASH; h += STG_BUILD_TPB) {
    keys[h] = -1;
    hsl[h] = -1;
    esl[h] = -1;
  }
  for (int h = t; h <= STG_SLOTS; h += STG_BUILD_TPB) s_hist[h] = 0;
  if (t == 0) {
    s_nh = 0;
    s_ne = 0;
    s_bad = 0;
  }
  __syncthreads();
  auto outside = [&](int j) { return j < rb0 || j >= rb1; };
  auto insert = [&](int j, bool halo) {
    unsigned h = stg_hash(j);
    for (int p = 0; p < STG_HASH; ++p, h = (h + 1) & (STG_HASH - 1)) {
      const int old = atomicCAS(&keys[h], -1, j);
      if (old == -1) {
        esl[h] = (short)min(atomicAdd(&s_ne, 1), 32767);
        if (halo) {
          const int x = atomicAdd(&s_nh, 1);
          hsl[h] = (short)min(x, 32767);
          if (x < FCG_HMAX) hrow[x] = j;
        }
        return;
      }
      if (old == j) return;
    }
    s_bad = 1;
  };
  auto find = [&](int j) {
    unsigned h = stg_hash(j);
    for (int p = 0; p < STG_HASH; ++p, h = (h + 1) & (STG_HASH - 1)) {
      const int k = keys[h];
      if (k == j) return (int)h;
      if (k == -1) break;
    }
    return -1;
  };
  // the halo: operator columns outside the block
  for (int l = t; l < nown; l += STG_BUILD_TPB)
    for (int e = rowptr[rb0 + l]; e < rowptr[rb0 + l + 1]; ++e)
      if (outside(col[e])) insert(col[e], true);
  __syncthreads();
  const int nh = s_nh;
  // the rest of the ext rows: M^-1 columns of the own and the halo rows
  for (int l = t; l < nown; l += STG_BUILD_TPB) {
    const int i = rb0 + l;
    for (int q = 0; q < mcnt[i]; ++q) {
      const int j = mcol[(size_t)q * mstride + i];
      if (outside(j)) insert(j, false);
    }
  }
  for (int x = t; x < min(nh, FCG_HMAX); x += STG_BUILD_TPB) {
    const int i = hrow[x];
    for (int q = 0; q < mcnt[i]; ++q) {
      const int j = mcol[(size_t)q * mstride + i];
      if (outside(j)) insert(j, false);
    }
  }
  __syncthreads();
  const int ne = s_ne;
  const int npos = nown + nh, ng = (npos + 31) / 32;
  if (s_bad || nh > FCG_HMAX || ne > STG_EXTMAX || ng > STG_MAXG) {
    if (t == 0) atomicAnd(stat, 0);
    return;
  }
  // the row at unsorted position p (own rows, then halo rows)
  auto pos_row = [&](int p) { return p < nown ? rb0 + p : hrow[p - nown]; };
  // positions ordered by entry count, longest first (counting sort)
  for (int p = t; p < npos; p += STG_BUILD_TPB) {
    const int m = mcnt[pos_row(p)];
    if (m > STG_SLOTS)
      s_bad = 1;
    else
      atomicAdd(&s_hist[m], 1);
  }
  __syncthreads();
  if (t == 0) {
    int off = 0;
    for (int m = STG_SLOTS; m >= 0; --m) {
      const int c = s_hist[m];
      s_hist[m] = off;
      off += c;
    }
  }
  __syncthreads();
  if (s_bad) {
    if (t == 0) atomicAnd(stat, 0);
    return;
  }
  for (int p = t; p < npos; p += STG_BUILD_TPB) prow[atomicAdd(&s_hist[mcnt[pos_row(p)]], 1)] = p;
  __syncthreads();
  // the row at sorted position q (-1: padding)
  auto srow = [&](int q) { return q < npos ? pos_row(prow[q]) : -1; };
  // groups of 32 positions: slots = the longest row
  for (int g = wid; g < ng; g += STG_BUILD_TPB / 32) {
    const int i = srow(g * 32 + lane);
    int m = i >= 0 ? mcnt[i] : 0;
    m = __reduce_max_sync(0xffffffffu, m);
    if (lane == 0) s_gsl[g] = m;
  }
  __syncthreads();
  if (t == 0) {
    int off = 0;
    for (int g = 0; g < ng; ++g) {
      s_goff[g] = off;
      off += s_gsl[g] * 32;
    }
    s_total = off;
    if (off > STG_ENTRIES) s_bad = 1;
  }
  __syncthreads();
  if (s_bad) {
    if (t == 0) atomicAnd(stat, 0);
    return;
  }
  // the staging index of column j (own rows first, then the ext rows)
  auto sidx = [&](int j) -> int {
    if (!outside(j)) return j - rb0;
    const int h = find(j);
    return h < 0 ? 0 : rpb + esl[h];
  };
  for (int h = t; h < STG_HASH; h += STG_BUILD_TPB)
    if (keys[h] >= 0) im.ext[esl[h]] = keys[h];
  for (int x = t; x < nh; x += STG_BUILD_TPB) im.hrow[x] = hrow[x];
  for (int q = t; q < npos; q += STG_BUILD_TPB) {
    const int p = prow[q];
    const int i = pos_row(p);
    im.pridx[q] = (unsigned short)sidx(i);
    im.puidx[q] = (unsigned short)(p < nown ? p : rpb + (p - nown));
    im.pm[q] = (unsigned char)mcnt[i];
    im.pmd[q] = mdiag[i];
    im.pdnv[q] = (float)dinv[i];
  }
  for (int q = t; q < ng * 32; q += STG_BUILD_TPB) {
    const int i = srow(q);
    const int m = i >= 0 ? mcnt[i] : 0;
    const int base = s_goff[q >> 5] + (q & 31);
    for (int z = 0; z < s_gsl[q >> 5]; ++z) {
      const bool have = z < m;
      im.sidx[base + z * 32] = (unsigned short)(have ? sidx(mcol[(size_t)z * mstride + i]) : 0);
      im.sval[base + z * 32] = have ? mval[(size_t)z * mstride + i] : 0.f;
    }
  }
  // the operator's columns, remapped to the staged u
  for (int l = t; l < nown; l += STG_BUILD_TPB)
    for (int e = rowptr[rb0 + l]; e < rowptr[rb0 + l + 1]; ++e) {
      const int j = col[e];
      int r = j - rb0;
      if (outside(j)) {
        const int h = find(j);
        r = h < 0 ? 0 : rpb + hsl[h];
      }
      remap[e] = r;
    }
  for (int g = t; g < ng; g += STG_BUILD_TPB) {
    im.goff[g] = s_goff[g];
    im.gsl[g] = s_gsl[g];
  }
  if (t == 0) {
    im.npos = npos;
    im.ne = ne;
    im.nh = nh;
    im.total = s_total;
    atomicMax(stat + 1, nh);
    atomicMax(stat + 2, ne);
    atomicMax(stat + 3, s_total);
  }
}

// The one-hop M^-1 rows with the entries in registers (up to MREG, compared
// and placed by unrolled loops instead of a local-memory array); the same
// entries, values and order as k_build_minv.  A row with more entries is
// flagged in `over` and built by k_build_minv afterwards.
constexpr int MREG = 24;
__global__ void __launch_bounds__(128) k_build_minv_reg(int n, const int* __restrict__ rowptr,
                                                        const int* __restrict__ col, const float* __restrict__ gd,
                                                        const float* __restrict__ gl, const int* __restrict__ rev,
                                                        const float* __restrict__ dh, float eps, int stride, int* mcnt,
                                                        int* mcol, float* mval, float* mdiag, int* over, int* mok,
                                                        int* stage_stat) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    // the status words of this build, before any later kernel updates them
    *mok = 1;
    stage_stat[0] = 1;
    stage_stat[1] = stage_stat[2] = stage_stat[3] = 0;
  }
  if (i >= n) return;
  int cols[MREG];
  float vals[MREG];
#pragma unroll
  for (int s = 0; s < MREG; ++s) {
    cols[s] = -1;
    vals[s] = 0.f;
  }
  int m = 0;
  float dsum = 0.f;
  bool full = false;
  auto add = [&](int j, float v) {
    if (j == i) {
      dsum += v;
      return;
    }
    bool found = false;
#pragma unroll
    for (int s = 0; s < MREG; ++s)
      if (cols[s] == j) {
        vals[s] += v;
        found = true;
      }
    if (!found) {
      if (m < MREG) {
#pragma unroll
        for (int s = 0; s < MREG; ++s)
          if (s == m) {
            cols[s] = j;
            vals[s] = v;
          }
        ++m;
      } else {
        full = true;
      }
    }
  };
  auto row_k = [&](int k, float gki) {
    add(k, gki * gd[k]);
    for (int k2 = rowptr[k]; k2 < rowptr[k + 1]; ++k2)
      if (col[k2] < k) add(col[k2], gki * gl[k2]);
  };
  row_k(i, gd[i]);
  for (int kk = rowptr[i]; kk < rowptr[i + 1]; ++kk) {
    const int u = col[kk];
    if (u > i && rev[kk] >= 0) row_k(u, gl[rev[kk]]);
  }
  over[i] = full ? 1 : 0;
  if (full) return;
  const float di = dh[i];
#pragma unroll
  for (int s = 0; s < MREG; ++s)
    if (s < m) {
      mcol[(size_t)s * stride + i] = cols[s];
      mval[(size_t)s * stride + i] = di * vals[s] * dh[cols[s]];
    }
  mcnt[i] = m;
  mdiag[i] = di * (dsum + eps) * di;
}

// The factored form of the learned M^-1 (SolverDev::mfac) from the factor:
// row i's lower entries (j < i, G_ij = gl at the operator entry) and the
// entries of column i (G_ki for the operator's k > i, at the reverse entry of
// row k), in the operator's order.
__global__ void k_build_gfac(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                             const float* __restrict__ gd, const float* __restrict__ gl, const int* __restrict__ rev,
                             int stride, int* mcnt, int* mcol, float* mval, float* mdiag, int* mok) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) *mok = 1;
  if (i >= n) return;
  int nl = 0, nu = 0;
  for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
    const int j = col[k];
    if (j < i) {
      mcol[(size_t)nl * stride + i] = j;
      mval[(size_t)nl * stride + i] = gl[k];
      ++nl;
    } else if (j > i && rev[k] >= 0) {
      const size_t e = (size_t)(LV_MAX_EDGES + nu) * stride + i;
      mcol[e] = j;
      mval[e] = gl[rev[k]];
      ++nu;
    }
  }
  mcnt[i] = nl | (nu << 8);
  mdiag[i] = gd[i];
}

// ---------------------------------------------------------------------------
// Streaming mixed-precision solve for systems beyond the register-resident
// solver (k_big): the refinement and the single-reduction CG of k_fcg, with
// the operator read in the mesh's slot-major face layout (column = the face's
// neighbour m.fnbr[k*cap + i], FP32 and FP64 weights per slot, written by the
// assembly) and every vector in global memory.  One 1024-thread block per SM;
// block b owns the contiguous rows [b*rpb, (b+1)*rpb), thread t the rows
// rb0 + t + k*1024, so every vector pass is coalesced.  Neighbour values move
// through point-to-point exchanges (a block waits only for the blocks whose
// rows its rows reference, from a mask built once per operator), dot products
// through grid-wide phases.  A Jacobi iteration makes two passes over the
// rows (w = A u with the dots; the vector updates with u = D^-1 r), one
// exchange and one phase; a learned one a third pass (u = M^-1 r from the
// explicit slot-major M^-1) and a second exchange.  The FP64 correction
// x += sigma d of a refinement step is never exchanged: the next residual
// pass reads x_j + sigma d_j of every neighbour, and the owners fold the
// correction into x after the phase that ends that pass.
// ---------------------------------------------------------------------------
constexpr int BIG_TPB = 1024;
constexpr int BIG_SB = 8;    // slots loaded together (FP32 passes)
constexpr int BIG_SB64 = 4;  // (FP64 residual)
constexpr int BIG_MASK_WORDS = FCG_MAX_BLOCKS / 32;

struct BigArgs {
  int n, nb, rpb, cap;        // cap: slot stride of the face arrays
  const int* nf;              // faces per row
  const int* fcol;            // slot-major neighbour index
  const float* w32e;          // slot-major weights, FP32 and FP64
  const double* w64e;
  const float* dg32;          // the reference's diagonal term (FP32)
  const float* dinv32;        // 1 / (diag + sum_j w_ij) (FP32)
  const double* diag;
  const double* b;
  double* x;
  double* r64;
  float *r, *u, *w, *p, *s, *d;
  const int* mcnt;            // learned M^-1: off-diagonal count, slot-major entries, diagonal
  const int* mcol;
  const float* mval;
  const float* mdiag;
  int mstride;
  const int* minv_ok;
  int learned;
  int mfac;                   // M^-1 in factored form (SolverDev::mfac): D^-1/2 = dh, G's entries, eps
  const float* dh;
  float eps;
  float* y;                   // G D^-1/2 r of the factored form
  const unsigned* masks;      // [nb][BIG_MASK_WORDS] blocks whose rows a block references
  unsigned long long* slots;  // partial words [2 parities][RG_WORDS][nb]
  unsigned* counter;
  unsigned* sync_base;
  unsigned* flags;
  int* status;
  double tol2;
  int itmax;
  long long spin;
  const int* nonsingular;
  int sg_mode;                // as FcgArgs
  double* pprev;
  double* bprev;
  const float* sgD;
  float* sgstore;
  const double* sgcoef;
  int* jref;
  int* out_iters;
  int* out_outer;
  int* out_method;
  double* out_d;
  long long* counters;
};

// Blocks whose rows the operator's (and with M^-1 also M^-1's) rows of each
// block reference: one block per solve block, bit j of mask[b] for block j.
__global__ void __launch_bounds__(BIG_TPB) k_big_masks(int n, int rpb, int cap, const int* __restrict__ nf,
                                                       const int* __restrict__ fcol, const int* __restrict__ mcnt,
                                                       const int* __restrict__ mcol, int mstride,
                                                       unsigned* masks) {
  __shared__ unsigned sm[BIG_MASK_WORDS];
  for (int t = threadIdx.x; t < BIG_MASK_WORDS; t += blockDim.x) sm[t] = 0u;
  __syncthreads();
  const int me = blockIdx.x;
  const int rb0 = me * rpb, rb1 = min(n, rb0 + rpb);
  auto mark = [&](int j) {
    const int bj = j / rpb;
    if (bj != me) atomicOr(&sm[bj >> 5], 1u << (bj & 31));
  };
  for (int i = rb0 + (int)threadIdx.x; i < rb1; i += blockDim.x) {
    const int m = nf[i];
    for (int k = 0; k < m; ++k) mark(fcol[(size_t)k * cap + i]);
    if (mcnt) {
      const int q = mcnt[i];
      for (int k = 0; k < q; ++k) mark(mcol[(size_t)k * mstride + i]);
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < BIG_MASK_WORDS; t += blockDim.x) masks[(size_t)me * BIG_MASK_WORDS + t] = sm[t];
}

// Row i's FP32 difference-form product dg_i v_i + sum_k w_k (v_i - v_j).
// The face count and the first BIG_SB slots (columns and weights) are loaded
// together: slots below LV_MAX_EDGES lie inside the arrays whatever the row's
// count, and a slot past it (a stale value) only selects the row itself and
// is not added.  Then the gathers of the neighbours' values.
__device__ __forceinline__ float big_row32(const BigArgs& a, int i, float vi, const float* __restrict__ v) {
  const int nfi = ld_nc(a.nf + i);
  int jj[BIG_SB];
  float wv[BIG_SB], xv[BIG_SB];
#pragma unroll
  for (int q = 0; q < BIG_SB; ++q) {
    jj[q] = ld_nc(a.fcol + (size_t)q * a.cap + i);
    wv[q] = ld_nc(a.w32e + (size_t)q * a.cap + i);
  }
  float acc = ld_nc(a.dg32 + i) * vi;
#pragma unroll
  for (int q = 0; q < BIG_SB; ++q) xv[q] = __ldcg(v + (q < nfi ? jj[q] : i));
#pragma unroll
  for (int q = 0; q < BIG_SB; ++q)
    if (q < nfi) acc = fmaf(wv[q], vi - xv[q], acc);
  for (int k = BIG_SB; k < nfi; ++k) {
    const size_t e = (size_t)k * a.cap + i;
    acc = fmaf(ld_nc(a.w32e + e), vi - __ldcg(v + ld_nc(a.fcol + e)), acc);
  }
  return acc;
}

// Row i's FP64 residual b_i - (diag_i x_i + sum_k w_k (x_i - x_j)), the slots
// in the same order (the columns of the first BIG_SB slots loaded with the
// face count, the weights and gathers BIG_SB64 at a time).
__device__ __forceinline__ double big_res64(const BigArgs& a, int i, double bi) {
  const int nfi = ld_nc(a.nf + i);
  int jj[BIG_SB];
#pragma unroll
  for (int q = 0; q < BIG_SB; ++q) jj[q] = ld_nc(a.fcol + (size_t)q * a.cap + i);
  const double xi = __ldcg(a.x + i);
  double acc = ld_nc(a.diag + i) * xi;
#pragma unroll
  for (int h = 0; h < BIG_SB; h += BIG_SB64) {
    if (h >= nfi) break;
    double wv[BIG_SB64], xv[BIG_SB64];
#pragma unroll
    for (int q = 0; q < BIG_SB64; ++q) {
      wv[q] = ld_nc(a.w64e + (size_t)(h + q) * a.cap + i);
      xv[q] = __ldcg(a.x + (h + q < nfi ? jj[h + q] : i));
    }
#pragma unroll
    for (int q = 0; q < BIG_SB64; ++q)
      if (h + q < nfi) acc += wv[q] * (xi - xv[q]);
  }
  for (int k = BIG_SB; k < nfi; ++k) {
    const size_t e = (size_t)k * a.cap + i;
    acc += ld_nc(a.w64e + e) * (xi - __ldcg(a.x + ld_nc(a.fcol + e)));
  }
  return bi - acc;
}

// Row i of u = M^-1 r: md_i r_i + the row's slots in order, BIG_SB at a time.
// The slot loads wait for the row's count and stop at its last slot (a
// speculative chunk past the count cost more DRAM traffic than the round
// trip it saves: M^-1 rows have about 18 entries, so whole unused slot lines
// were fetched).
__device__ __forceinline__ float big_mrow(const BigArgs& a, int i, const float* __restrict__ r) {
  const int mc = a.mcnt[i];
  float acc = a.mdiag[i] * __ldcg(r + i);
  for (int k0 = 0; k0 < mc; k0 += BIG_SB) {
    int jj[BIG_SB];
    float mv[BIG_SB], rv[BIG_SB];
#pragma unroll
    for (int q = 0; q < BIG_SB; ++q) {
      const size_t e = (size_t)min(k0 + q, mc - 1) * a.mstride + i;
      jj[q] = ld_nc(a.mcol + e);
      mv[q] = ld_nc(a.mval + e);
    }
#pragma unroll
    for (int q = 0; q < BIG_SB; ++q) rv[q] = __ldcg(r + jj[q]);
#pragma unroll
    for (int q = 0; q < BIG_SB; ++q)
      if (k0 + q < mc) acc = fmaf(mv[q], rv[q], acc);
  }
  return acc;
}

constexpr int BIG_GB = 4;  // entries of a factored M^-1 pass loaded together (rows have ~3)

// The factored M^-1, first pass: row i of y = G z, z = D^-1/2 r (G's lower
// entries of the row; z_j of a neighbour formed from its exchanged r).
__device__ __forceinline__ float big_grow(const BigArgs& a, int i, const float* __restrict__ r) {
  const int nl = ld_nc(a.mcnt + i) & 0xff;
  float acc = ld_nc(a.mdiag + i) * (ld_nc(a.dh + i) * __ldcg(r + i));
  for (int k0 = 0; k0 < nl; k0 += BIG_GB) {
    int jj[BIG_GB];
    float mv[BIG_GB], zv[BIG_GB];
#pragma unroll
    for (int q = 0; q < BIG_GB; ++q) {
      const size_t e = (size_t)min(k0 + q, nl - 1) * a.mstride + i;
      jj[q] = ld_nc(a.mcol + e);
      mv[q] = ld_nc(a.mval + e);
    }
#pragma unroll
    for (int q = 0; q < BIG_GB; ++q) zv[q] = ld_nc(a.dh + jj[q]) * __ldcg(r + jj[q]);
#pragma unroll
    for (int q = 0; q < BIG_GB; ++q)
      if (k0 + q < nl) acc = fmaf(mv[q], zv[q], acc);
  }
  return acc;
}

// Second pass: row i of u = D^-1/2 (G^T y + eps z) (the entries G_ki of
// column i, from the exchanged y of the rows k > i).
__device__ __forceinline__ float big_gtrow(const BigArgs& a, int i, const float* __restrict__ r,
                                           const float* __restrict__ y) {
  const int nu = ld_nc(a.mcnt + i) >> 8;
  const float di = ld_nc(a.dh + i);
  float acc = ld_nc(a.mdiag + i) * __ldcg(y + i);
  for (int k0 = 0; k0 < nu; k0 += BIG_GB) {
    int jj[BIG_GB];
    float mv[BIG_GB], yv[BIG_GB];
#pragma unroll
    for (int q = 0; q < BIG_GB; ++q) {
      const size_t e = (size_t)(LV_MAX_EDGES + min(k0 + q, nu - 1)) * a.mstride + i;
      jj[q] = ld_nc(a.mcol + e);
      mv[q] = ld_nc(a.mval + e);
    }
#pragma unroll
    for (int q = 0; q < BIG_GB; ++q) yv[q] = __ldcg(y + jj[q]);
#pragma unroll
    for (int q = 0; q < BIG_GB; ++q)
      if (k0 + q < nu) acc = fmaf(mv[q], yv[q], acc);
  }
  return di * fmaf(a.eps, di * __ldcg(r + i), acc);
}

template <bool LEARNED>
__global__ void __launch_bounds__(BIG_TPB, 1) k_big(BigArgs a) {
  constexpr int TPB = BIG_TPB;
  const int n = a.n;
  const int rb0 = blockIdx.x * a.rpb;
  const int rb1 = min(n, rb0 + a.rpb);
  const int t = threadIdx.x;
  float* __restrict__ vr = a.r;
  float* __restrict__ vu = a.u;
  float* __restrict__ vw = a.w;
  float* __restrict__ vp = a.p;
  float* __restrict__ vs = a.s;
  float* __restrict__ vd = a.d;
  __shared__ unsigned s_mask[BIG_MASK_WORDS];
  if (t == 0) {
    s_base[0] = __ldcg(a.sync_base);
    s_base[1] = __ldcg(a.sync_base + 1);
  }
  for (int q = t; q < BIG_MASK_WORDS; q += TPB) s_mask[q] = __ldcg(a.masks + (size_t)blockIdx.x * BIG_MASK_WORDS + q);
  __syncthreads();
  const bool learned0 = LEARNED && a.learned != 0 && *a.minv_ok != 0;
  unsigned ep = 0, xe = 0;
  bool ok = true;
  double bmean = 0.0;
  if (*a.nonsingular == 0) {
    // singular operator: b projected to zero mean
    double v[1] = {0.0}, tt[1];
    for (int i = rb0 + t; i < rb1; i += TPB) v[0] += a.b[i];
    ok = fphase<1, double>(a, ++ep, v, tt);
    __shared__ double s_mean;
    if (t == 0) s_mean = tt[0] / (double)n;
    __syncthreads();
    bmean = s_mean;
  }
  // the sweep's start (own rows): P and b kept for the next sweep, the last
  // sweep's change stored, and with a shift P moved to the Galerkin start;
  // the neighbours see the shifted P after the exchange
  if (ok && a.sg_mode) {
    const double c0 = a.sg_mode == 2 ? a.sgcoef[0] : 0.0, c1 = a.sg_mode == 2 ? a.sgcoef[1] : 0.0;
    for (int i = rb0 + t; i < rb1; i += TPB) {
      const double p0 = a.x[i], pv = a.pprev[i];
      if (a.sgstore) a.sgstore[i] = (float)(p0 - pv);
      a.pprev[i] = p0;
      a.bprev[i] = a.b[i];
      if (a.sg_mode == 2) a.x[i] = sweep_shift(p0, pv, a.sgD ? (double)a.sgD[i] : 0.0, c0, c1);
    }
    if (a.sg_mode == 2) ok = nexchange(a, ++xe, s_mask);
  }
  const int jref = *a.jref;
  const int capit = jref > 0 ? jref : a.itmax;
  bool learned = learned0;
  int it = 0, updates = 0;
  double bnorm2 = 0.0, rtrue2 = 0.0;
  float gam_old = 1.f, alpha = 1.f;
  bool fall = false;
  // u = M^-1 r: the exchange of r, then the explicit M^-1 rows, or the
  // factored form's two passes with the exchange of y between them
  auto mpass = [&]() -> bool {
    if (!nexchange(a, ++xe, s_mask)) return false;
    if (a.mfac) {
      for (int i = rb0 + t; i < rb1; i += TPB) a.y[i] = big_grow(a, i, vr);
      if (!nexchange(a, ++xe, s_mask)) return false;
      for (int i = rb0 + t; i < rb1; i += TPB) vu[i] = big_gtrow(a, i, vr, a.y);
    } else {
      for (int i = rb0 + t; i < rb1; i += TPB) vu[i] = big_mrow(a, i, vr);
    }
    return true;
  };
  while (ok) {
    // ---- FP64 residual b - A x (difference form)
    double v2[2] = {0.0, 0.0}, t2[2];
    for (int i = rb0 + t; i < rb1; i += TPB) {
      const double bi = a.b[i] - bmean;
      const double ri = big_res64(a, i, bi);
      a.r64[i] = ri;
      v2[0] += ri * ri;
      v2[1] += bi * bi;
    }
    if (!(ok = fphase<2, double>(a, ++ep, v2, t2))) break;
    rtrue2 = t2[0];
    bnorm2 = t2[1];
    if (rtrue2 <= a.tol2 * bnorm2 || it >= a.itmax || updates >= FCG_MAX_UPDATES) break;
    __shared__ double s_sig[2];
    __shared__ float s_rho_upd;
    if (t == 0) {
      const double sg = sqrt(rtrue2);
      s_sig[0] = sg;
      s_sig[1] = 1.0 / sg;
      s_rho_upd = fmaxf(FCG_UPDATE_DROP * FCG_UPDATE_DROP, (float)(0.25 * a.tol2 * bnorm2 / rtrue2));
    }
    __syncthreads();
    const double sigma = s_sig[0], inv_sigma = s_sig[1];
    const float rho_upd = s_rho_upd;
    ++updates;
    if (fall) {
      learned = false;
      fall = false;
    }
    // restart: r = r64 / sigma, u = M^-1 r
    for (int i = rb0 + t; i < rb1; i += TPB) {
      const float ri = (float)(a.r64[i] * inv_sigma);
      vr[i] = ri;
      if (!learned) vu[i] = a.dinv32[i] * ri;
    }
    if (learned && !(ok = mpass())) break;
    bool first = true;  // p, s, d start from zero (never read)
    while (true) {
      if (!(ok = nexchange(a, ++xe, s_mask))) break;
      // w = A u (FP32 difference form) with the dots (r,u), (w,u), (r,r)
      float v3[3] = {0.f, 0.f, 0.f}, t3[3];
      for (int i = rb0 + t; i < rb1; i += TPB) {
        const float ui = __ldcg(vu + i), ri = __ldcg(vr + i);
        const float acc = big_row32(a, i, ui, vu);
        vw[i] = acc;
        v3[0] = fmaf(ri, ui, v3[0]);
        v3[1] = fmaf(acc, ui, v3[1]);
        v3[2] = fmaf(ri, ri, v3[2]);
      }
      if (!(ok = fphase<3, float>(a, ++ep, v3, t3))) break;
      const float gam = t3[0], delta = t3[1], rho = t3[2];
      if (rho <= rho_upd || it >= a.itmax || !(delta > 0.f)) break;
      if (learned && it >= capit) {
        fall = true;
        break;
      }
      const float beta = first ? 0.f : gam / gam_old;
      alpha = first ? gam / delta : gam / (delta - beta * gam / alpha);
      // two rows per round, every load issued before the stores
      for (int i = rb0 + t; i < rb1; i += 2 * TPB) {
        const int i2 = i + TPB;
        const bool on2 = i2 < rb1;
        const int k2 = on2 ? i2 : i;
        float ui[2], wi[2], pi[2], si[2], di[2], ri[2], dv[2];
        ui[0] = __ldcg(vu + i), ui[1] = __ldcg(vu + k2);
        wi[0] = __ldcg(vw + i), wi[1] = __ldcg(vw + k2);
        ri[0] = __ldcg(vr + i), ri[1] = __ldcg(vr + k2);
        if (!first) {
          pi[0] = __ldcg(vp + i), pi[1] = __ldcg(vp + k2);
          si[0] = __ldcg(vs + i), si[1] = __ldcg(vs + k2);
          di[0] = __ldcg(vd + i), di[1] = __ldcg(vd + k2);
        }
        if (!learned) dv[0] = a.dinv32[i], dv[1] = a.dinv32[k2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          pi[h] = first ? ui[h] : fmaf(beta, pi[h], ui[h]);
          si[h] = first ? wi[h] : fmaf(beta, si[h], wi[h]);
          di[h] = first ? alpha * pi[h] : fmaf(alpha, pi[h], di[h]);
          ri[h] = fmaf(-alpha, si[h], ri[h]);
        }
        vp[i] = pi[0], vs[i] = si[0], vd[i] = di[0], vr[i] = ri[0];
        if (!learned) vu[i] = dv[0] * ri[0];
        if (on2) {
          vp[i2] = pi[1], vs[i2] = si[1], vd[i2] = di[1], vr[i2] = ri[1];
          if (!learned) vu[i2] = dv[1] * ri[1];
        }
      }
      gam_old = gam;
      first = false;
      ++it;
      if (learned && !(ok = mpass())) break;
    }
    if (!ok) break;
    // the correction: x += sigma d on the own rows, then the neighbours' x
    // for the next residual
    if (!first) {
      for (int i = rb0 + t; i < rb1; i += TPB) a.x[i] += sigma * (double)__ldcg(vd + i);
      if (!(ok = nexchange(a, ++xe, s_mask))) break;
    }
  }
  if (ok && blockIdx.x == 0 && t == 0) {
    a.sync_base[0] = s_base[0] + ep * (unsigned)a.nb;
    a.sync_base[1] = s_base[1] + xe;
    *a.out_iters = it;
    *a.out_outer = updates;
    *a.out_method = learned ? LV_METHOD_LEARNED_PCG : LV_METHOD_MIXED_IR;
    if (!a.learned) *a.jref = it;
    a.out_d[0] = rtrue2;
    a.out_d[1] = bnorm2;
    a.out_d[2] = rtrue2;
    count_solve(a.counters, it, rtrue2, bnorm2, rtrue2, a.tol2);
  }
}

// ---------------------------------------------------------------------------
// MINRES (Paige & Saunders, SIAM J. Numer. Anal. 12, 1975) in FP64 without a
// preconditioner: the reference's default pressure solve, Krylov.jl's
// minres! with atol = rtol = tol (pressure.jl:219-220).  The recurrences and
// stopping tests are the oracle's restatement's: phibar = ||r|| <= atol +
// rtol ||r0||, or ||A r|| / (||A|| ||r||) <= rtol (an inconsistent singular
// system), or a Lanczos breakdown (beta = 0).  A persistent kernel over the
// operator's CSR; each iteration makes two passes, each ending in a
// grid-wide phase (alpha = (v, y), then beta^2 = (y, y)), and one pass over
// the own rows for the direction and the iterate.  The Lanczos vector v =
// y / beta of a neighbour is formed from its y where it is gathered, so no
// neighbour exchange is needed; the scalar recurrences run once per block.
// ---------------------------------------------------------------------------
constexpr int MR_TPB = 1024;
constexpr int MR_EB = 4;  // entries loaded together

struct MinresArgs {
  int n, nb, rpb;   // n: unknowns (ncomp per particle, interleaved); rpb: unknowns per block
  int ncomp;        // 1: the pressure; 2: the two velocity components of the viscous system
  int eform;        // 0: y_i = diag_i v_i + sum_e w_e (v_i - v_j) (PressureOperator, pressure.jl:119-130);
                    // 1: y_i = sum_e w_e v_j, then + diag_i v_i (ThreadedMat mul!, viscous_solver.jl:12-22)
  const int* rowptr;
  const int* col;
  const double* w;
  const double* diag;
  const double* b;
  double* x;
  double* lz[2];  // the Lanczos vectors r1, r2 (roles swap every iteration)
  double* dw[3];  // the directions w, w1, w2 (roles rotate every iteration)
  unsigned long long* slots;
  unsigned* counter;
  unsigned* sync_base;
  int* status;
  long long spin;
  double atol, rtol, tol2;
  int itmax;
  int* out_iters;
  int* out_solved;
  int* out_method;
  double* out_d;
  long long* counters;
};

// Row r of A v with v = sc * src (unknown r is component c of particle i),
// in the operator's form (eform), the entries in order, MR_EB loads at a time
__device__ __forceinline__ double mr_apply(const MinresArgs& a, int r, const double* src, double sc, double vi) {
  const int i = a.ncomp == 1 ? r : r >> 1, c = r - i * a.ncomp;
  const int e0 = a.rowptr[i], e1 = a.rowptr[i + 1];
  double acc = a.eform ? 0.0 : a.diag[i] * vi;
  for (int b0 = e0; b0 < e1; b0 += MR_EB) {
    int j[MR_EB];
    double wv[MR_EB], xv[MR_EB];
#pragma unroll
    for (int q = 0; q < MR_EB; ++q) {
      const int e = min(b0 + q, e1 - 1);
      j[q] = ld_nc(a.col + e);
      wv[q] = ld_nc(a.w + e);
    }
#pragma unroll
    for (int q = 0; q < MR_EB; ++q) xv[q] = sc * __ldcg(src + (size_t)a.ncomp * j[q] + c);
#pragma unroll
    for (int q = 0; q < MR_EB; ++q)
      if (b0 + q < e1) acc += a.eform ? wv[q] * xv[q] : wv[q] * (vi - xv[q]);
  }
  if (a.eform) acc += a.diag[i] * vi;
  return acc;
}

__global__ void __launch_bounds__(MR_TPB, 1) k_minres(MinresArgs a) {
  const int n = a.n, t = threadIdx.x;
  const int rb0 = blockIdx.x * a.rpb, rb1 = min(n, rb0 + a.rpb);
  if (t == 0) {
    s_base[0] = __ldcg(a.sync_base);
    s_base[1] = __ldcg(a.sync_base + 1);
  }
  __syncthreads();
  unsigned ep = 0;
  // the scalar recurrences, formed by thread 0 of every block from the
  // phases' totals (bit-identical in all blocks, so all take the same exits)
  __shared__ double sc[16];
  enum { BETA, OLDB, DBAR, EPSLN, PHIBAR, CS, SN, TNORM2, S, ALFA, PHI, DENOM, OLDEPS, DELTA, TOL, BB };
  __shared__ int s_stop;
  // r1 = b - A x (x as given), r2 = r1, w = w2 = 0; beta1 = ||r1||
  double* R1 = a.lz[0];
  double* R2 = a.lz[1];
  double v2[2] = {0.0, 0.0}, t2[2];
  for (int i = rb0 + t; i < rb1; i += MR_TPB) {
    const double xi = __ldcg(a.x + i);
    const double bi = a.b[i];
    const double r = bi - mr_apply(a, i, a.x, 1.0, xi);
    R1[i] = r;
    R2[i] = r;
    a.dw[0][i] = 0.0;
    a.dw[2][i] = 0.0;
    v2[0] += r * r;
    v2[1] += bi * bi;
  }
  bool ok = fphase<2, double>(a, ++ep, v2, t2);
  if (t == 0) {
    const double beta1 = sqrt(t2[0]);
    sc[BETA] = beta1;
    sc[OLDB] = 0.0;
    sc[DBAR] = 0.0;
    sc[EPSLN] = 0.0;
    sc[PHIBAR] = beta1;
    sc[CS] = -1.0;
    sc[SN] = 0.0;
    sc[TNORM2] = 0.0;
    sc[TOL] = a.atol + a.rtol * beta1;
    sc[BB] = t2[1];
    s_stop = beta1 == 0.0 ? 2 : 0;  // 2: solved
  }
  __syncthreads();
  int itn = 0;
  int wi = 0;  // w = dw[wi], w1 = dw[(wi + 1) % 3], w2 = dw[(wi + 2) % 3] before the rotation
  while (ok && s_stop == 0 && itn < a.itmax) {
    ++itn;
    const double beta = sc[BETA], oldb = sc[OLDB];
    if (t == 0) sc[S] = 1.0 / beta;
    __syncthreads();
    const double s = sc[S];
    // y = A v - (beta / oldb) r1 with v = s r2 (the neighbours' v from their r2)
    const double c1 = itn >= 2 ? beta / oldb : 0.0;
    double va[1] = {0.0}, ta[1];
    for (int i = rb0 + t; i < rb1; i += MR_TPB) {
      const double vi = s * __ldcg(R2 + i);
      double y = mr_apply(a, i, R2, s, vi);
      if (itn >= 2) y -= c1 * R1[i];
      R1[i] = y;
      va[0] += vi * y;
    }
    if (!(ok = fphase<1, double>(a, ++ep, va, ta))) break;
    // y -= (alfa / beta) r2; then r1 <- r2, r2 <- y; beta^2 = (y, y)
    const double c2 = ta[0] / beta;
    double vb[1] = {0.0}, tb[1];
    for (int i = rb0 + t; i < rb1; i += MR_TPB) {
      const double y = R1[i] - c2 * R2[i];
      R1[i] = y;
      vb[0] += y * y;
    }
    if (!(ok = fphase<1, double>(a, ++ep, vb, tb))) break;
    if (t == 0) {
      const double eps = 2.220446049250313e-16;
      const double alfa = ta[0];
      const double ob = beta;
      const double nb = sqrt(tb[0]);
      sc[OLDB] = ob;
      sc[BETA] = nb;
      sc[TNORM2] += alfa * alfa + ob * ob + nb * nb;
      const double oldeps = sc[EPSLN];
      const double delta = sc[CS] * sc[DBAR] + sc[SN] * alfa;
      const double gbar = sc[SN] * sc[DBAR] - sc[CS] * alfa;
      sc[EPSLN] = sc[SN] * nb;
      sc[DBAR] = -sc[CS] * nb;
      const double root = sqrt(gbar * gbar + sc[DBAR] * sc[DBAR]);
      const double gamma = fmax(sqrt(gbar * gbar + nb * nb), eps);
      sc[CS] = gbar / gamma;
      sc[SN] = nb / gamma;
      sc[PHI] = sc[CS] * sc[PHIBAR];
      sc[PHIBAR] = sc[SN] * sc[PHIBAR];
      sc[DENOM] = 1.0 / gamma;
      sc[OLDEPS] = oldeps;
      sc[DELTA] = delta;
      const double rnorm = sc[PHIBAR], anorm = sqrt(sc[TNORM2]), arnorm = sc[PHIBAR] * root;
      int st = 0;
      if (rnorm <= sc[TOL]) st = 2;
      else if (anorm > 0 && rnorm > 0 && arnorm / (anorm * rnorm) <= a.rtol) st = 2;
      else if (nb == 0.0) st = 2;
      s_stop = st;
    }
    __syncthreads();
    // w1 <- w2, w2 <- w, w = (v - oldeps w1 - delta w2) denom; x += phi w,
    // with v = s r2 (r2 before its swap below)
    wi = (wi + 1) % 3;
    double* Wn = a.dw[wi];             // the new w (the old w1's buffer)
    double* Wm1 = a.dw[(wi + 1) % 3];  // w1: the old w2
    double* Wm2 = a.dw[(wi + 2) % 3];  // w2: the old w
    const double phi = sc[PHI], denom = sc[DENOM], oldeps = sc[OLDEPS], delta = sc[DELTA];
    for (int i = rb0 + t; i < rb1; i += MR_TPB) {
      const double vi = s * R2[i];
      const double wv = (vi - oldeps * Wm1[i] - delta * Wm2[i]) * denom;
      Wn[i] = wv;
      a.x[i] += phi * wv;
    }
    // r1 <- r2, r2 <- y
    double* tmp = R1;
    R1 = R2;
    R2 = tmp;
  }
  // the true residual of the final iterate
  double vr[1] = {0.0}, tr[1] = {0.0};
  if (ok) {
    for (int i = rb0 + t; i < rb1; i += MR_TPB) {
      const double xi = a.x[i];
      const double r = a.b[i] - mr_apply(a, i, a.x, 1.0, xi);
      vr[0] += r * r;
    }
    ok = fphase<1, double>(a, ++ep, vr, tr);
  }
  if (ok && blockIdx.x == 0 && t == 0) {
    a.sync_base[0] = s_base[0] + ep * (unsigned)a.nb;
    const int solved = s_stop == 2 ? 1 : 0;
    *a.out_iters = itn;
    *a.out_solved = solved;
    *a.out_method = LV_METHOD_MINRES;
    a.out_d[0] = tr[0];
    a.out_d[1] = sc[BB];
    a.out_d[2] = tr[0];
    a.counters[0] += 1;
    a.counters[1] += itn;
    if (!solved) a.counters[2] += 1;
  }
}

int g_big_blocks_per_sm[2] = {-1, -1};

int g_fcg_blocks_per_sm[2] = {-1, -1};
int g_fcg_halo_blocks_per_sm[2] = {-1, -1};

// blocks and rows per thread of the flag-reduced solve of n rows: one block
// per SM while one row per thread suffices, else two rows per thread, then
// two blocks per SM
void fcg_shape(const lv_ctx* c, int n, int* nb, int* R) {
  *nb = c->num_sms;
  *R = 1;
  if (n > *nb * FCG_TPB) *R = 2;
  if (n > *nb * FCG_TPB * 2) *nb = std::min(c->num_sms * 2, FCG_MAX_BLOCKS);
}

// whether the staged mode's shared memory leaves nb blocks co-resident (the
// shared-memory attributes were set per device by lv_fcg_device_setup; the
// occupancy is the same on every device of this kind)
bool stage_fits(const lv_ctx* c, int nb, int R) {
  static std::once_flag once;
  std::call_once(once, []() {
    int b1 = 0, b2 = 0;
    const int bytes = (int)sizeof(StageSmem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b1, k_fcg<1, true>, FCG_TPB, bytes) != cudaSuccess) b1 = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b2, k_fcg<2, true>, FCG_TPB, bytes) != cudaSuccess) b2 = 0;
    cudaGetLastError();
    g_fcg_halo_blocks_per_sm[0] = b1;
    g_fcg_halo_blocks_per_sm[1] = b2;
  });
  return g_fcg_halo_blocks_per_sm[R - 1] * c->num_sms >= nb;
}



}  // namespace

// The staged solve's and its image builder's shared memory on the current device.
int lv_fcg_device_setup() {
  const int bytes = (int)sizeof(StageSmem);
  cudaError_t e = cudaFuncSetAttribute(k_fcg<1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_fcg<2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_stage_build, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)STG_BUILD_SMEM);
  return e == cudaSuccess ? LV_OK : LV_ERR_CUDA;
}

// Rows the flag-reduced solver holds (one or two blocks per SM, two rows per
// thread at most); larger systems use the streaming solver.
int lv_fcg_capacity(lv_ctx* c) {
  if (g_fcg_blocks_per_sm[0] < 0) {
    int b1 = 0, b2 = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b1, k_fcg<1, false>, FCG_TPB, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b2, k_fcg<2, false>, FCG_TPB, 0);
    g_fcg_blocks_per_sm[0] = b1;
    g_fcg_blocks_per_sm[1] = b2;
  }
  if (g_fcg_blocks_per_sm[1] < 1) return 0;
  const int per_sm = std::min(g_fcg_blocks_per_sm[1], 2);
  return std::min(c->num_sms * per_sm, FCG_MAX_BLOCKS) * FCG_TPB * 2;
}

static int ensure_minv(lv_ctx* c) {
  SolverDev& sv = c->sv;
  const int rows = c->cap;
  if (sv.mrows >= rows && sv.mcnt) return LV_OK;
  cudaFree(sv.mcnt);
  cudaFree(sv.mcol);
  cudaFree(sv.mval);
  cudaFree(sv.mdiag);
  cudaFree(sv.mok);
  cudaFree(sv.stage);
  cudaFree(sv.remap);
  cudaFree(sv.stage_stat);
  sv.mcnt = nullptr;
  sv.mcol = nullptr;
  sv.mval = nullptr;
  sv.mdiag = nullptr;
  sv.mok = nullptr;
  sv.stage = nullptr;
  sv.remap = sv.stage_stat = nullptr;
  sv.stage_ready = false;
  sv.mrows = 0;
  const int maxb = std::min(c->num_sms * 2, FCG_MAX_BLOCKS);
  bool ok = cudaMalloc(&sv.mcnt, sizeof(int) * rows) == cudaSuccess;
  ok = ok && cudaMalloc(&sv.mcol, sizeof(int) * (size_t)MMAX * rows) == cudaSuccess;
  ok = ok && cudaMalloc(&sv.mval, sizeof(float) * (size_t)MMAX * rows) == cudaSuccess;
  ok = ok && cudaMalloc(&sv.mdiag, sizeof(float) * rows) == cudaSuccess;
  ok = ok && cudaMalloc(&sv.mok, sizeof(int)) == cudaSuccess;
  ok = ok && cudaMalloc(&sv.stage, sizeof(StageImage) * (size_t)maxb) == cudaSuccess;
  ok = ok && cudaMalloc(&sv.remap, sizeof(int) * (size_t)LV_MAX_EDGES * rows) == cudaSuccess;
  ok = ok && cudaMalloc(&sv.stage_stat, sizeof(int) * 4) == cudaSuccess;
  if (!ok) return lv_fail(c, LV_ERR_CUDA, "allocation of the learned preconditioner matrix failed");
  cudaMemsetAsync(sv.mok, 0, sizeof(int), c->stream);
  cudaMemsetAsync(sv.stage_stat, 0, sizeof(int) * 4, c->stream);
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
  cudaFree(sv.stage);
  cudaFree(sv.remap);
  cudaFree(sv.stage_stat);
  sv.mcnt = nullptr;
  sv.mcol = nullptr;
  sv.mval = nullptr;
  sv.mdiag = nullptr;
  sv.mok = nullptr;
  sv.stage = nullptr;
  sv.remap = sv.stage_stat = nullptr;
  sv.stage_ready = false;
  sv.mrows = 0;
}

// Largest per-block halo of the last built factor (0: staged mode off).
int lv_fcg_halo_info(lv_ctx* c, int* max_rows) {
  *max_rows = c->sv.stage_ready ? c->sv.stage_max[0] : 0;
  return LV_OK;
}

// Builds the explicit learned M^-1 from the current factor (after
// lv_learn_factor_current).
int lv_fcg_build_minv(lv_ctx* c) {
  const int n = c->n;
  if (int rc = ensure_minv(c)) return rc;
  c->big_masks_valid = false;  // the streaming solver's masks cover M^-1's pattern
  const float *gd, *gl, *dh, *gl2;
  const int *rev, *rowptr2, *col2, *rev2;
  lv_learn_factor_ptrs(c, &gd, &gl, &dh, &rev);
  lv_learn_factor2_ptrs(c, &rowptr2, &col2, &gl2, &rev2);
  if (!gd) return lv_fail(c, LV_ERR_BAD_ARGUMENT, "learned solve without a factor");
  // systems beyond the staged solver take the factored form (one-hop factor)
  c->sv.mfac = !rowptr2 && n > lv_fcg_capacity(c);
  c->sv.stage_ready = false;
  if (c->sv.mfac) {
    k_build_gfac<<<lv_blocks(n, 256), 256, 0, c->stream>>>(n, c->sv.rowptr, c->sv.col, gd, gl, rev, c->sv.mrows,
                                                           c->sv.mcnt, c->sv.mcol, c->sv.mval, c->sv.mdiag, c->sv.mok);
    LV_LAUNCH_CHECK(c, "k_build_gfac");
    return LV_OK;
  }
  if (rowptr2) {
    const int one = 1;
    cudaMemcpyAsync(c->sv.mok, &one, sizeof(int), cudaMemcpyHostToDevice, c->stream);
    const int init[4] = {1, 0, 0, 0};
    cudaMemcpyAsync(c->sv.stage_stat, init, sizeof(init), cudaMemcpyHostToDevice, c->stream);
    k_build_minv<<<lv_blocks(n, 128), 128, 0, c->stream>>>(n, c->sv.rowptr, c->sv.col, gd, gl, rev, rowptr2, col2,
                                                            gl2, rev2, dh, c->learn_eps, c->sv.mrows, c->sv.mcnt,
                                                            c->sv.mcol, c->sv.mval, c->sv.mdiag, c->sv.mok, nullptr);
    LV_LAUNCH_CHECK(c, "k_build_minv");
  } else {
    // rows of up to MREG entries in registers, the rest (flagged) as before
    int* over = c->sv.remap;  // scratch: the staged image build rewrites it below
    k_build_minv_reg<<<lv_blocks(n, 128), 128, 0, c->stream>>>(n, c->sv.rowptr, c->sv.col, gd, gl, rev, dh,
                                                                c->learn_eps, c->sv.mrows, c->sv.mcnt, c->sv.mcol,
                                                                c->sv.mval, c->sv.mdiag, over, c->sv.mok,
                                                                c->sv.stage_stat);
    LV_LAUNCH_CHECK(c, "k_build_minv_reg");
    k_build_minv<<<lv_blocks(n, 128), 128, 0, c->stream>>>(n, c->sv.rowptr, c->sv.col, gd, gl, rev, nullptr, nullptr,
                                                            nullptr, nullptr, dh, c->learn_eps, c->sv.mrows,
                                                            c->sv.mcnt, c->sv.mcol, c->sv.mval, c->sv.mdiag,
                                                            c->sv.mok, over);
    LV_LAUNCH_CHECK(c, "k_build_minv");
  }
  // the staged image of every solve block, for the shape lv_fcg_solve
  // launches; the host learns whether every image fit (one synchronisation
  // per factor)
  const char* env = getenv("LVGPU_FCG_HALO");
  c->fcg_halo = !(env && env[0] == '0');
  c->sv.stage_ready = false;
  int nb, R;
  fcg_shape(c, n, &nb, &R);
  if (n <= lv_fcg_capacity(c) && c->fcg_halo && stage_fits(c, nb, R) &&
      nb <= std::min(c->num_sms * 2, FCG_MAX_BLOCKS)) {
    // (stage_stat was initialised by the first kernel of the M^-1 build)
    k_stage_build<<<nb, STG_BUILD_TPB, STG_BUILD_SMEM, c->stream>>>(
        n, (n + nb - 1) / nb, c->sv.rowptr, c->sv.col, c->sv.mcnt, c->sv.mcol, c->sv.mval, c->sv.mdiag, c->sv.dinv,
        c->sv.mrows, static_cast<StageImage*>(c->sv.stage), c->sv.remap, c->sv.stage_stat);
    LV_LAUNCH_CHECK(c, "k_stage_build");
    int st[4] = {0, 0, 0, 0}, mok = 0;
    cudaMemcpyAsync(st, c->sv.stage_stat, sizeof(st), cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(&mok, c->sv.mok, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    if (int rc = lv_cuda_check(c, cudaStreamSynchronize(c->stream), "k_stage_build")) return rc;
    c->sv.stage_ready = st[0] != 0 && mok != 0;
    for (int q = 0; q < 3; ++q) c->sv.stage_max[q] = st[q + 1];
  }
  return LV_OK;
}

// Launches the flag-reduced mixed-precision solve into x (device), stats into
// the given slot.  Returns LV_ERR_BAD_ARGUMENT when the system is too large.
int lv_fcg_solve(lv_ctx* c, double* x, int slot, bool learned) {
  const int n = c->n;
  const int capn = lv_fcg_capacity(c);
  if (n > capn || n < 1) return LV_ERR_BAD_ARGUMENT;
  if (learned && !c->sv.mcnt) return lv_fail(c, LV_ERR_BAD_ARGUMENT, "learned solve without a preconditioner");
  int nb, R;
  fcg_shape(c, n, &nb, &R);
  if (g_fcg_blocks_per_sm[R - 1] * c->num_sms < nb) return LV_ERR_BAD_ARGUMENT;
  FcgArgs a;
  a.n = n;
  a.nb = nb;
  a.rows_per_block = (n + nb - 1) / nb;
  a.rowptr = c->sv.rowptr;
  a.col = c->sv.col;
  a.w = c->sv.w;
  a.w32 = c->sv.w32;
  a.dg32 = c->sv.d32;
  a.dinv32 = c->sv.dinv32;
  a.diag = c->sv.diag;
  a.dinv = c->sv.dinv;
  a.b = c->sv.b;
  a.x = x;
  a.rbuf = c->sv.r32;
  a.rtag = c->sv.rtag;
  a.sg_mode = 0;
  a.pprev = c->sv.pprev;
  a.bprev = c->sv.bprev;
  a.sgD = nullptr;
  a.sgstore = nullptr;
  a.sgcoef = c->sv.sgomega;
  if (c->sg_pending && c->sg_P == x) {
    a.sg_mode = c->sg_shift ? 2 : 1;
    a.sgD = c->sg_D;
    a.sgstore = c->sg_store;
    c->sg_pending = false;
  }
  a.ubuf = c->sv.f32a;
  a.slots = c->sv.fslots;
  a.counter = c->sv.bar + 2;
  a.sync_base = reinterpret_cast<unsigned*>(c->sv.iters + LV_IT_FCG_BASE);
  a.flags = reinterpret_cast<unsigned*>(c->sv.fslots + 8192);
  a.status = c->status;
  a.tol2 = c->tol * c->tol;
  a.itmax = c->itmax;
  a.spin = c->spin_limit;
  a.nonsingular = c->sv.iters + LV_IT_NONSINGULAR;
  a.learned = learned ? 1 : 0;
  a.mcnt = c->sv.mcnt;
  a.mcol = c->sv.mcol;
  a.mval = c->sv.mval;
  a.mdiag = c->sv.mdiag;
  a.mstride = c->sv.mrows;
  a.minv_ok = learned ? c->sv.mok : c->sv.iters + LV_IT_NONSINGULAR;  // read only in learned mode
  const bool halo = learned && c->sv.stage_ready && stage_fits(c, nb, R);
  a.stage = static_cast<const StageImage*>(c->sv.stage);
  a.remap = c->sv.remap;
  a.jref = c->sv.iters + LV_IT_JREF + slot;  // the same sweep of the last Jacobi mixed solve
  a.out_iters = c->sv.iters + slot;
  a.out_outer = c->sv.iters + LV_IT_OUTER + slot;
  a.out_method = c->sv.iters + LV_IT_METHOD + slot;
  a.out_d = c->sv.dstats + 3 * slot;
  a.counters = c->sv.counters;
  if (c->fcg_reset) {
    // first launch, or a launch after a failed one: the counter, the flags
    // (all FCG_MAX_BLOCKS of them) and the bases start from zero
    cudaMemsetAsync(a.counter, 0, sizeof(unsigned), c->stream);
    cudaMemsetAsync(a.flags, 0, sizeof(unsigned) * FLAG_STRIDE * FCG_MAX_BLOCKS, c->stream);
    cudaMemsetAsync(a.sync_base, 0, sizeof(unsigned) * 2, c->stream);
    cudaMemsetAsync(a.rtag, 0, sizeof(unsigned long long) * (size_t)c->cap, c->stream);
    c->fcg_reset = false;
  }
  void* args[] = {&a};
  const void* fn = halo ? (R == 1 ? (const void*)k_fcg<1, true> : (const void*)k_fcg<2, true>)
                        : (R == 1 ? (const void*)k_fcg<1, false> : (const void*)k_fcg<2, false>);
  const size_t dyn = halo ? sizeof(StageSmem) : 0;
  cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(nb), dim3(FCG_TPB), args, dyn, c->stream);
  c->launches++;
  if (e != cudaSuccess) {
    c->fcg_reset = true;
    return lv_cuda_check(c, e, "k_fcg cooperative launch");
  }
  return LV_OK;
}

// ------------------------------------------------------- streaming solver

namespace {
constexpr int BIG_SLOT_OFF = 64;                                  // u32 words: counter, bases, then partials
constexpr int BIG_FLAG_OFF = BIG_SLOT_OFF + 2 * RG_WORDS * FCG_MAX_BLOCKS;
constexpr int BIG_SYNC_WORDS = BIG_FLAG_OFF + FLAG_STRIDE * FCG_MAX_BLOCKS;

template <class T>
T* big_alloc(lv_ctx* c, size_t count, bool* ok) {
  void* p = nullptr;
  if (cudaMalloc(&p, sizeof(T) * std::max<size_t>(count, 1)) != cudaSuccess) {
    *ok = false;
    return nullptr;
  }
  c->allocs.push_back(p);  // freed with the context
  return static_cast<T*>(p);
}

int big_blocks(lv_ctx* c, bool learned) {
  int& b = g_big_blocks_per_sm[learned ? 1 : 0];
  if (b < 0) {
    int v = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, learned ? (const void*)k_big<true> : (const void*)k_big<false>,
                                                  BIG_TPB, 0);
    b = v;
  }
  return b >= 1 ? std::min(c->num_sms, FCG_MAX_BLOCKS) : 0;
}
}  // namespace

int lv_big_prepare(lv_ctx* c) {
  SolverDev& sv = c->sv;
  if (sv.ew32) return LV_OK;
  const size_t cap = (size_t)c->cap;
  bool ok = true;
  sv.ew32 = big_alloc<float>(c, (size_t)LV_MAX_EDGES * cap, &ok);
  sv.ew64 = big_alloc<double>(c, (size_t)LV_MAX_EDGES * cap, &ok);
  sv.bvec = big_alloc<float>(c, 7 * cap, &ok);
  sv.br64 = big_alloc<double>(c, cap, &ok);
  sv.bmasks = big_alloc<unsigned>(c, (size_t)FCG_MAX_BLOCKS * BIG_MASK_WORDS, &ok);
  sv.bsync = big_alloc<unsigned>(c, BIG_SYNC_WORDS, &ok);
  if (!ok) {
    sv.ew32 = nullptr;
    sv.ew64 = nullptr;
    return lv_fail(c, LV_ERR_CUDA, "allocation of the streaming solver's buffers failed");
  }
  c->big_reset = true;
  c->big_masks_valid = false;
  return LV_OK;
}

// Launches the streaming mixed-precision solve into x (device), stats into
// the given slot.
int lv_big_solve(lv_ctx* c, double* x, int slot, bool learned) {
  const int n = c->n;
  SolverDev& sv = c->sv;
  if (!sv.ew32) return lv_fail(c, LV_ERR_NOT_MESHED, "streaming solve of an operator assembled without its buffers");
  if (learned && !sv.mcnt) return lv_fail(c, LV_ERR_BAD_ARGUMENT, "learned solve without a preconditioner");
  const int nb = big_blocks(c, learned);
  if (nb < 1) return lv_fail(c, LV_ERR_CUDA, "the streaming solver does not fit an SM");
  const int rpb = (n + nb - 1) / nb;
  // the explicit M^-1 reaches two hops; the operator and the factored form one
  const bool need_m = learned && !sv.mfac;
  if (!c->big_masks_valid || (need_m && !c->big_masks_m)) {
    // the neighbour blocks of every block: the operator's pattern, and M^-1's
    // for an explicit learned solve (a superset serves a Jacobi solve too)
    k_big_masks<<<nb, BIG_TPB, 0, c->stream>>>(n, rpb, c->m.cap, c->m.nfaces, c->m.fnbr, need_m ? sv.mcnt : nullptr,
                                               sv.mcol, sv.mrows, sv.bmasks);
    LV_LAUNCH_CHECK(c, "k_big_masks");
    c->big_masks_valid = true;
    c->big_masks_m = need_m;
  }
  BigArgs a;
  a.n = n;
  a.nb = nb;
  a.rpb = rpb;
  a.cap = c->m.cap;
  a.nf = c->m.nfaces;
  a.fcol = c->m.fnbr;
  a.w32e = sv.ew32;
  a.w64e = sv.ew64;
  a.dg32 = sv.d32;
  a.dinv32 = sv.dinv32;
  a.diag = sv.diag;
  a.b = sv.b;
  a.x = x;
  a.r64 = sv.br64;
  const size_t cap = (size_t)c->cap;
  a.r = sv.bvec;
  a.u = sv.bvec + cap;
  a.w = sv.bvec + 2 * cap;
  a.p = sv.bvec + 3 * cap;
  a.s = sv.bvec + 4 * cap;
  a.d = sv.bvec + 5 * cap;
  a.mcnt = sv.mcnt;
  a.mcol = sv.mcol;
  a.mval = sv.mval;
  a.mdiag = sv.mdiag;
  a.mstride = sv.mrows;
  a.minv_ok = learned ? sv.mok : sv.iters + LV_IT_NONSINGULAR;  // read only in learned mode
  a.learned = learned ? 1 : 0;
  a.mfac = (learned && sv.mfac) ? 1 : 0;
  a.dh = nullptr;
  a.eps = c->learn_eps;
  a.y = sv.bvec + 6 * cap;
  if (a.mfac) {
    const float *gd, *gl;
    const int* rev;
    lv_learn_factor_ptrs(c, &gd, &gl, &a.dh, &rev);
  }
  a.masks = sv.bmasks;
  a.counter = sv.bsync;
  a.sync_base = sv.bsync + 1;
  a.slots = reinterpret_cast<unsigned long long*>(sv.bsync + BIG_SLOT_OFF);
  a.flags = sv.bsync + BIG_FLAG_OFF;
  a.status = c->status;
  a.tol2 = c->tol * c->tol;
  a.itmax = c->itmax;
  a.spin = c->spin_limit;
  a.nonsingular = sv.iters + LV_IT_NONSINGULAR;
  a.sg_mode = 0;
  a.pprev = sv.pprev;
  a.bprev = sv.bprev;
  a.sgD = nullptr;
  a.sgstore = nullptr;
  a.sgcoef = sv.sgomega;
  if (c->sg_pending && c->sg_P == x) {
    a.sg_mode = c->sg_shift ? 2 : 1;
    a.sgD = c->sg_D;
    a.sgstore = c->sg_store;
    c->sg_pending = false;
  }
  a.jref = sv.iters + LV_IT_JREF + slot;
  a.out_iters = sv.iters + slot;
  a.out_outer = sv.iters + LV_IT_OUTER + slot;
  a.out_method = sv.iters + LV_IT_METHOD + slot;
  a.out_d = sv.dstats + 3 * slot;
  a.counters = sv.counters;
  if (c->big_reset) {
    cudaMemsetAsync(sv.bsync, 0, sizeof(unsigned) * BIG_SYNC_WORDS, c->stream);
    c->big_reset = false;
  }
  void* args[] = {&a};
  const void* fn = learned ? (const void*)k_big<true> : (const void*)k_big<false>;
  cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(nb), dim3(BIG_TPB), args, 0, c->stream);
  c->launches++;
  if (e != cudaSuccess) {
    c->big_reset = true;
    return lv_cuda_check(c, e, "k_big cooperative launch");
  }
  return LV_OK;
}

// ------------------------------------------------------------------ MINRES

// MINRES on the operator (rowptr, col, w, diag) of ncomp unknowns per
// particle in the given form, right-hand side b, iterate x, tolerances as the
// reference's minres! (atol = rtol = tol); statistics into `slot`.
static int minres_launch(lv_ctx* c, const int* rowptr, const int* col, const double* w, const double* diag,
                         const double* b, double* x, int ncomp, int eform, double tol, int itmax, int slot);

int lv_minres_solve(lv_ctx* c, double* x, int slot) {
  return minres_launch(c, c->sv.rowptr, c->sv.col, c->sv.w, c->sv.diag, c->sv.b, x, 1, 0, c->tol, c->itmax, slot);
}

static int minres_launch(lv_ctx* c, const int* rowptr, const int* col, const double* w, const double* diag,
                         const double* b, double* x, int ncomp, int eform, double tol, int itmax, int slot) {
  SolverDev& sv = c->sv;
  const int n = c->n * ncomp;
  static std::once_flag once;
  static int per_sm = 0;
  std::call_once(once, []() {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_minres, MR_TPB, 0) != cudaSuccess) per_sm = 0;
  });
  if (per_sm < 1) return lv_fail(c, LV_ERR_CUDA, "the MINRES kernel does not fit an SM");
  if (!sv.mrvec) {
    bool ok = true;
    sv.mrvec = big_alloc<double>(c, 10 * (size_t)c->cap, &ok);  // five vectors of up to 2 cap unknowns
    sv.mrsync = big_alloc<unsigned>(c, BIG_SLOT_OFF + 2 * RG_WORDS * FCG_MAX_BLOCKS, &ok);
    if (!ok) {
      sv.mrvec = nullptr;
      return lv_fail(c, LV_ERR_CUDA, "allocation of the MINRES vectors failed");
    }
    c->mr_reset = true;
  }
  const int nb = std::max(1, std::min(std::min(c->num_sms, FCG_MAX_BLOCKS), lv_blocks(n, 64)));
  MinresArgs a;
  a.n = n;
  a.nb = nb;
  a.rpb = (n + nb - 1) / nb;
  a.ncomp = ncomp;
  a.eform = eform;
  a.rowptr = rowptr;
  a.col = col;
  a.w = w;
  a.diag = diag;
  a.b = b;
  a.x = x;
  const size_t cap = 2 * (size_t)c->cap;
  a.lz[0] = sv.mrvec;
  a.lz[1] = sv.mrvec + cap;
  a.dw[0] = sv.mrvec + 2 * cap;
  a.dw[1] = sv.mrvec + 3 * cap;
  a.dw[2] = sv.mrvec + 4 * cap;
  a.counter = sv.mrsync;
  a.sync_base = sv.mrsync + 1;
  a.slots = reinterpret_cast<unsigned long long*>(sv.mrsync + BIG_SLOT_OFF);
  a.status = c->status;
  a.spin = c->spin_limit;
  a.atol = tol;
  a.rtol = tol;
  a.tol2 = tol * tol;
  a.itmax = itmax;
  a.out_iters = sv.iters + slot;
  a.out_solved = sv.iters + LV_IT_OUTER + slot;
  a.out_method = sv.iters + LV_IT_METHOD + slot;
  a.out_d = sv.dstats + 3 * slot;
  a.counters = sv.counters;
  if (c->mr_reset) {
    cudaMemsetAsync(sv.mrsync, 0, sizeof(unsigned) * (BIG_SLOT_OFF + 2 * RG_WORDS * FCG_MAX_BLOCKS), c->stream);
    c->mr_reset = false;
  }
  void* args[] = {&a};
  cudaError_t e = cudaLaunchCooperativeKernel((const void*)k_minres, dim3(nb), dim3(MR_TPB), args, 0, c->stream);
  c->launches++;
  if (e != cudaSuccess) {
    c->mr_reset = true;
    return lv_cuda_check(c, e, "k_minres cooperative launch");
  }
  return LV_OK;
}

int lv_minres_general(lv_ctx* c, const int* rowptr, const int* col, const double* w, const double* diag,
                      const double* b, double* x, int ncomp, int eform, double tol, int itmax, int slot) {
  return minres_launch(c, rowptr, col, w, diag, b, x, ncomp, eform, tol, itmax, slot);
}
