// Learned preconditioner for the pressure solve: a message-passing network
// over the Voronoi adjacency graph that emits a sparse factor G on the
// pattern of the lower triangle of the pressure operator, so that
//     M^-1 = D^-1/2 (Gt^T Gt + eps I) D^-1/2,   G = Gt D^-1/2
// is SPD (D = diagonal of the operator).  The network works on the
// Jacobi-normalised operator At = D^-1/2 A D^-1/2 = I - What:
//
//   X     node features [1, diag/adiag, sum_j what_ij, max_j what_ij, deg/8,
//         sum_{j<i} what_ij, #{j<i}/8, max_{j<i} what_ij, 0...] (16)
//   H1    = relu([X,  Agg X ] W0 + b0)            Agg(H)_i = sum_j what_ij H_j
//   H2    = H1 + relu([H1, Agg H1] W1 + b1)
//   H3    = H2 + relu([H2, Agg H2] W2 + b2)        (3 layers, hidden width 32)
//   Gt_ii = 1 + H3_i . rd
//   Gt_ij = what_ij sum_c ro_c H3_ic H3_jc          for j < i, j ~ i
//   Gt_ij = pw_ij sum_c ro2_c H3_ic H3_jc           for j < i at distance two
//                                                   (two-hop pattern, optional)
// with the path weight pw_ij = sum_k what_ik what_kj over common neighbours.
//
// The matrix products of the layers run on the tensor cores with BF16
// operands and FP32 accumulation: the forward [N x 32|64] x [32|64 x 32] (the
// factor of every timestep) and the training's backward dX = dZ W^T and
// dW = X^T dZ as tcgen05.mma into tensor memory; everything else is FP32.  Training minimises either the exact FSAI (Kaporin) objective
//     (1/N) [ tr(Gt At Gt^T) - 2 sum_i log Gt_ii ]
// (Kolotilina & Yeremin, SIAM J. Matrix Anal. Appl. 14, 1993; Kaporin,
// Numer. Linear Algebra Appl. 1, 1994), whose minimiser on the pattern is the
// FSAI factor, or a Hutchinson estimate of
//     || Gt At Gt^T - I ||_F^2 / N = E_z || Gt At Gt^T z - z ||^2 / N,
// z Rademacher, whose gradient with respect to each entry (a, b) of Gt is
// 2 (r_a t_b + z_a s_b), r = Gt At Gt^T z - z, t = At Gt^T z, s = At Gt^T r.
// Backward kernels are written by hand; Adam updates the FP32 master weights.
#include <cuda_bf16.h>
#include <math.h>

#include <algorithm>
#include <vector>

#include "lv_internal.cuh"

namespace {

constexpr int HID = 32;
constexpr int FIN = 16;
constexpr int KC0 = 2 * FIN;  // 32
constexpr int KC = 2 * HID;   // 64
constexpr int OFF_W0 = 0;
constexpr int OFF_B0 = OFF_W0 + KC0 * HID;
constexpr int OFF_W1 = OFF_B0 + HID;
constexpr int OFF_B1 = OFF_W1 + KC * HID;
constexpr int OFF_W2 = OFF_B1 + HID;
constexpr int OFF_B2 = OFF_W2 + KC * HID;
constexpr int OFF_RD = OFF_B2 + HID;
constexpr int OFF_RO = OFF_RD + HID;
constexpr int OFF_RO2 = OFF_RO + HID;  // readout of the two-hop entries
constexpr int NPARAM = OFF_RO2 + HID;
constexpr int Q2MAX = 40;  // two-hop (not one-hop) neighbours kept per row
constexpr int WBF_W0 = 0, WBF_W1 = KC0 * HID, WBF_W2 = KC0 * HID + KC * HID, NWBF = KC0 * HID + 2 * KC * HID;
constexpr int MAXPROBES = 8;
constexpr int PART_BLOCKS = 304;
constexpr int BW_BLOCKS = 608;  // backward layers: four blocks on each of 152 SMs
constexpr int RB_BLOCKS = 1216;  // readout backward: eight blocks on each of 152 SMs

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat16 a = __float2bfloat16_rn(lo), b = __float2bfloat16_rn(hi);
  return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

// ---------------------------------------------------------------- preparation

__global__ void k_lprep_dh(int n, const double* __restrict__ adiag, float* dh) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dh[i] = (float)(1.0 / sqrt(adiag[i]));
}

// what_k = w_k dh_i dh_j; rev_k = position of (j, i) in row j; node features.
__global__ void k_lprep(int n, const int* __restrict__ rowptr, const int* __restrict__ col, const double* __restrict__ w,
                        const double* __restrict__ diag, const double* __restrict__ adiag,
                        const float* __restrict__ dh, float* what, int* rev, float* X) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int a = rowptr[i], b = rowptr[i + 1];
  const float dhi = dh[i];
  float s = 0.f, m = 0.f, sl = 0.f, ml = 0.f;
  int nl = 0;
  // entries eight at a time, and each neighbour's row searched eight entries
  // at a time (indexes clamped), so that the loads of a round overlap
  constexpr int EB = 8;
  for (int kb = a; kb < b; kb += EB) {
    int jj[EB], r0[EB], r1[EB];
    double wv[EB];
    float dj[EB];
#pragma unroll
    for (int u = 0; u < EB; ++u) {
      const int k = min(kb + u, b - 1);
      jj[u] = ld_nc(col + k);
      wv[u] = ld_nc(w + k);
    }
#pragma unroll
    for (int u = 0; u < EB; ++u) {
      dj[u] = ld_nc(dh + jj[u]);
      r0[u] = ld_nc(rowptr + jj[u]);
      r1[u] = ld_nc(rowptr + jj[u] + 1);
    }
#pragma unroll
    for (int u = 0; u < EB; ++u) {
      const int k = kb + u;
      if (k >= b) break;
      const int j = jj[u];
      const float v = (float)wv[u] * dhi * dj[u];
      what[k] = v;
      s += v;
      m = fmaxf(m, v);
      if (j < i) {
        sl += v;
        ml = fmaxf(ml, v);
        ++nl;
      }
      int r = -1;
      for (int t0 = r0[u]; t0 < r1[u] && r < 0; t0 += EB) {
        int cc[EB];
#pragma unroll
        for (int q = 0; q < EB; ++q) cc[q] = ld_nc(col + min(t0 + q, r1[u] - 1));
#pragma unroll
        for (int q = 0; q < EB; ++q)
          if (r < 0 && t0 + q < r1[u] && cc[q] == i) r = t0 + q;
      }
      rev[k] = r;
    }
  }
  float* x = X + (size_t)i * FIN;
  x[0] = 1.f;
  x[1] = (float)(diag[i] / adiag[i]);
  x[2] = s;
  x[3] = m;
  x[4] = (float)(b - a) * 0.125f;
  // the factor is lower-triangular in the index order: the lower neighbours
  x[5] = sl;
  x[6] = (float)nl * 0.125f;
  x[7] = ml;
#pragma unroll
  for (int f = 8; f < FIN; ++f) x[f] = 0.f;
}

// Two-hop pattern Q (j at distance exactly two from i, both triangles) as a
// CSR with the path weights pw_ij = sum_k what_ik what_kj and the transposed
// positions rev2; neighbours of neighbours in CSR order, at most Q2MAX per row.
__device__ int hop2_collect(int i, const int* __restrict__ rowptr, const int* __restrict__ col,
                            const float* __restrict__ what, int* qj, float* qw, int* overflow) {
  const int a = rowptr[i], b = rowptr[i + 1];
  int m = 0;
  for (int k1 = a; k1 < b; ++k1) {
    const int k = col[k1];
    const float wik = what[k1];
    for (int k2 = rowptr[k]; k2 < rowptr[k + 1]; ++k2) {
      const int j = col[k2];
      if (j == i) continue;
      bool one_hop = false;
      for (int t = a; t < b; ++t)
        if (col[t] == j) {
          one_hop = true;
          break;
        }
      if (one_hop) continue;
      int s = 0;
      while (s < m && qj[s] != j) ++s;
      if (s < m) {
        qw[s] = fmaf(wik, what[k2], qw[s]);
      } else if (m < Q2MAX) {
        qj[m] = j;
        qw[m] = wik * what[k2];
        ++m;
      } else {
        *overflow = 1;
      }
    }
  }
  return m;
}

__global__ void k_hop2_count(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                             const float* __restrict__ what, int* cnt, int* overflow) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int qj[Q2MAX];
  float qw[Q2MAX];
  int ov = 0;
  cnt[i] = hop2_collect(i, rowptr, col, what, qj, qw, &ov);
  if (ov) atomicOr(overflow, 1);
}

__global__ void k_hop2_fill(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                            const float* __restrict__ what, const int* __restrict__ rowptr2, int* col2, float* pw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int qj[Q2MAX];
  float qw[Q2MAX];
  int ov = 0;
  const int m = hop2_collect(i, rowptr, col, what, qj, qw, &ov);
  const int o = rowptr2[i];
  for (int s = 0; s < m; ++s) {
    col2[o + s] = qj[s];
    pw[o + s] = qw[s];
  }
}

__global__ void k_hop2_rev(int n, const int* __restrict__ rowptr2, const int* __restrict__ col2, int* rev2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int e = rowptr2[i]; e < rowptr2[i + 1]; ++e) {
    const int j = col2[e];
    int r = -1;
    for (int t = rowptr2[j]; t < rowptr2[j + 1]; ++t)
      if (col2[t] == i) {
        r = t;
        break;
      }
    rev2[e] = r;
  }
}

// ---------------------------------------------------------------- forward

// Feature rows stored as FP32 (training, whose backward pass reads them) or
// as BF16 (the per-step factor: the layer products take BF16 operands
// anyway, and half the bytes move).  A 16-byte chunk holds PER features.
template <typename T>
struct FeatIO;
template <>
struct FeatIO<float> {
  static constexpr int PER = 4;
  using Chunk = float4;
  __device__ static float get(const float4& c, int e) { return e == 0 ? c.x : (e == 1 ? c.y : (e == 2 ? c.z : c.w)); }
  // NB neighbours per round: their loads in flight together
  static constexpr int NB = 2;
};
template <>
struct FeatIO<__nv_bfloat16> {
  static constexpr int PER = 8;
  using Chunk = uint4;
  __device__ static float get(const uint4& c, int e) {
    const unsigned u = e < 2 ? c.x : (e < 4 ? c.y : (e < 6 ? c.z : c.w));
    return __uint_as_float((e & 1) ? (u & 0xffff0000u) : (u << 16));
  }
  static constexpr int NB = 4;
};

// 16 features of a row from registers
__device__ __forceinline__ void store_feat(float* p, const float (&h)[16]) {
  float4* q = reinterpret_cast<float4*>(p);
#pragma unroll
  for (int c = 0; c < 4; ++c) q[c] = make_float4(h[4 * c], h[4 * c + 1], h[4 * c + 2], h[4 * c + 3]);
}
__device__ __forceinline__ void store_feat(__nv_bfloat16* p, const float (&h)[16]) {
  uint4* q = reinterpret_cast<uint4*>(p);
#pragma unroll
  for (int c = 0; c < 2; ++c)
    q[c] = make_uint4(pack_bf16(h[8 * c], h[8 * c + 1]), pack_bf16(h[8 * c + 2], h[8 * c + 3]),
                      pack_bf16(h[8 * c + 4], h[8 * c + 5]), pack_bf16(h[8 * c + 6], h[8 * c + 7]));
}

// Row r's own features and aggregation Agg(Hin)_r = sum_k what_k Hin[col_k]
// for lane (r, half): half (l >> 4) of the KH features; rows past n give
// zeros.  FeatIO<T>::NB neighbours per round, their loads issued together;
// the sum runs over the neighbours in order.
template <int KH, typename T>
__device__ __forceinline__ void aggregate_row(int row, int half, int n, const T* __restrict__ Hin,
                                              const int* __restrict__ rowptr, const int* __restrict__ col,
                                              const float* __restrict__ what, float (&own)[KH / 2],
                                              float (&agg)[KH / 2]) {
  using IO = FeatIO<T>;
  using Chunk = typename IO::Chunk;
  constexpr int FH = KH / 2, PER = IO::PER, NC = FH / PER, NB = IO::NB;
  static_assert(FH % PER == 0, "16-byte feature chunks");
#pragma unroll
  for (int f = 0; f < FH; ++f) agg[f] = own[f] = 0.f;
  if (row >= n) return;
  {
    const Chunk* hr = reinterpret_cast<const Chunk*>(Hin + (size_t)row * KH + half * FH);
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      const Chunk v = hr[c];
#pragma unroll
      for (int e = 0; e < PER; ++e) own[c * PER + e] = IO::get(v, e);
    }
  }
  const int k1 = rowptr[row + 1];
  for (int k = rowptr[row]; k < k1; k += NB) {
    int jj[NB];
    float ww[NB];
#pragma unroll
    for (int u = 0; u < NB; ++u) {
      const int kk = min(k + u, k1 - 1);
      jj[u] = col[kk];
      ww[u] = what[kk];
    }
    Chunk ch[NB][NC];
#pragma unroll
    for (int u = 0; u < NB; ++u) {
      const Chunk* hj = reinterpret_cast<const Chunk*>(Hin + (size_t)jj[u] * KH + half * FH);
#pragma unroll
      for (int c = 0; c < NC; ++c) ch[u][c] = hj[c];
    }
#pragma unroll
    for (int u = 0; u < NB; ++u) {
      if (k + u >= k1) break;
#pragma unroll
      for (int c = 0; c < NC; ++c)
#pragma unroll
        for (int e = 0; e < PER; ++e) agg[c * PER + e] = fmaf(ww[u], IO::get(ch[u][c], e), agg[c * PER + e]);
    }
  }
}

// ---------------------------------------------------------------- forward on tcgen05
//
// Z = [Hin, Agg Hin] W + b;  Hout = (res ? Hin : 0) + relu(Z), in 128-row
// tiles on the fifth-generation tensor cores.  The tile's A operand
// (128 x K BF16) and W (K x 32 BF16, as its transpose: N x K) sit in shared
// memory in the canonical no-swizzle K-major layout: core matrices of 8 rows
// x 16 bytes, 128 bytes apart along K (LBO) and K x 16 bytes apart along the
// rows (SBO).  One thread issues K/16 tcgen05.mma (kind::f16, M = 128, N = 32,
// FP32 accumulation in tensor memory) and commits them to an mbarrier; each
// warp then reads its 32 rows of D with tcgen05.ld (thread = row, 32 columns)
// and writes Z and Hout as contiguous rows.
constexpr int TC_ROWS = 128;
constexpr int TC_TPB = 256;  // 8 warps: 16 rows each for the operand, a quarter of the lanes and half the columns of D each
constexpr unsigned TC_COLS = 32;  // tensor-memory columns (the minimum allocation)
constexpr long long TC_SPIN_LIMIT = 4000000000LL;  // cycles (about 2 s)

// byte offset of element (r, k) of a K-major operand with K columns
__device__ __forceinline__ int umma_off(int r, int k, int K) {
  return (r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}
// shared-memory matrix descriptor: start >> 4 [0,14), LBO >> 4 [16,30),
// SBO >> 4 [32,46), version 1 [46,48), no swizzle
__device__ __forceinline__ unsigned long long umma_desc(const void* p, unsigned lbo, unsigned sbo) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  return (unsigned long long)((a & 0x3FFFFu) >> 4) | ((unsigned long long)(lbo >> 4) << 16) |
         ((unsigned long long)(sbo >> 4) << 32) | (1ull << 46);
}
// instruction descriptor of kind::f16: D F32 [4,6), A BF16 [7,10), B BF16
// [10,13), both K-major, N >> 3 [17,23), M >> 4 [24,29)
constexpr unsigned TC_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(HID >> 3) << 17) |
                              ((unsigned)(TC_ROWS >> 4) << 24);

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ bool tc_bar_try(unsigned bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}
__device__ __forceinline__ bool tc_bar_wait(unsigned bar, unsigned parity) {
  const long long t0 = clock64();
  while (!tc_bar_try(bar, parity))
    if (clock64() - t0 > TC_SPIN_LIMIT) return false;
  return true;
}

// The A operand: the warp's 16 rows [Hin, Agg Hin] as BF16
// pairs at their K-major core-matrix positions (rows past n are zeros);
// with aggout, Agg Hin is also stored in FP32 (n x KH) for the backward
template <int KH, typename TIN>
__device__ void fill_xcat_umma(unsigned char* sA, int rl, int row0, int n, const TIN* __restrict__ Hin,
                               const int* __restrict__ rowptr, const int* __restrict__ col,
                               const float* __restrict__ what, float* aggout) {
  constexpr int K = 2 * KH, FH = KH / 2;
  const int lane = threadIdx.x & 31;
  const int r = lane & 15, half = lane >> 4;
  float own[FH], agg[FH];
  const int row = row0 + rl + r;
  aggregate_row<KH, TIN>(row, half, n, Hin, rowptr, col, what, own, agg);
  if (aggout && row < n) {
    float4* o = reinterpret_cast<float4*>(aggout + (size_t)row * KH + half * FH);
#pragma unroll
    for (int c4 = 0; c4 < FH / 4; ++c4) o[c4] = make_float4(agg[4 * c4], agg[4 * c4 + 1], agg[4 * c4 + 2], agg[4 * c4 + 3]);
  }
#pragma unroll
  for (int f = 0; f < FH; f += 2) {
    *reinterpret_cast<uint32_t*>(sA + umma_off(rl + r, half * FH + f, K)) = pack_bf16(own[f], own[f + 1]);
    *reinterpret_cast<uint32_t*>(sA + umma_off(rl + r, KH + half * FH + f, K)) = pack_bf16(agg[f], agg[f + 1]);
  }
}

template <int KH, typename TIN, typename TOUT>
__global__ void __launch_bounds__(TC_TPB, 4) k_layer_fwd(int n, const TIN* __restrict__ Hin,
                                                      const int* __restrict__ rowptr, const int* __restrict__ col,
                                                      const float* __restrict__ what,
                                                      const __nv_bfloat16* __restrict__ W,
                                                      const float* __restrict__ bias, int res, float* Z, TOUT* Hout,
                                                      float* Agg, int* status) {
  constexpr int K = 2 * KH;
  static_assert(K % 16 == 0, "K in steps of 16");
  __shared__ __align__(1024) unsigned char sA[TC_ROWS * K * 2];
  __shared__ __align__(1024) unsigned char sB[HID * K * 2];
  __shared__ __align__(8) unsigned long long s_bar;
  __shared__ unsigned s_tmem;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned bar = (unsigned)__cvta_generic_to_shared(&s_bar);
  // W^T into the B layout: element (n, k) = W[k][n]
  for (int t = threadIdx.x; t < K * HID; t += TC_TPB)
    *reinterpret_cast<__nv_bfloat16*>(sB + umma_off(t % HID, t / HID, K)) = W[t];
  if (warp == 0) {
    const unsigned holder = (unsigned)__cvta_generic_to_shared(&s_tmem);
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(holder), "r"(TC_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // B, for the tensor cores
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = s_tmem;
  const unsigned long long bdesc0 = umma_desc(sB, 128, K * 16);
  const unsigned long long adesc0 = umma_desc(sA, 128, K * 16);
  const int ntiles = (n + TC_ROWS - 1) / TC_ROWS;
  unsigned parity = 0;
  bool ok = true;
  for (int tl = blockIdx.x; tl < ntiles && ok; tl += gridDim.x) {
    const int row0 = tl * TC_ROWS;
    // A: each warp its 16 rows
    fill_xcat_umma<KH, TIN>(sA, warp * 16, row0, n, Hin, rowptr, col, what, Agg);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // A, for the tensor cores
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0) {
      tc_fence_after();
#pragma unroll
      for (int ks = 0; ks < K / 16; ++ks) {
        // K = 16 per instruction: two core matrices along K (256 bytes)
        const unsigned long long ad = adesc0 + (unsigned long long)((ks * 256) >> 4);
        const unsigned long long bd = bdesc0 + (unsigned long long)((ks * 256) >> 4);
        const unsigned acc = ks > 0 ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
                tmem),
            "l"(ad), "l"(bd), "r"(TC_IDESC), "r"(acc)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                   : "memory");
    }
    // the products (bounded wait; on a timeout a second bounded wait lets the
    // instructions in flight finish before the block gives up)
    const bool done = tc_bar_wait(bar, parity);
    if (!__syncthreads_and(done)) {
      if (threadIdx.x == 0) atomicOr(status, LV_FLAG_BARRIER_TIMEOUT);
      tc_bar_wait(bar, parity);
      ok = false;
      break;
    }
    parity ^= 1u;
    tc_fence_after();
    // warp w: lanes 32 (w % 4) .. + 31 (its quarter of tensor memory),
    // columns 16 (w / 4) .. + 15
    constexpr int DC = HID / 2;
    const int quarter = warp & 3, cb = (warp >> 2) * DC;
    uint32_t d[DC];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]), "=r"(d[6]), "=r"(d[7]),
          "=r"(d[8]), "=r"(d[9]), "=r"(d[10]), "=r"(d[11]), "=r"(d[12]), "=r"(d[13]), "=r"(d[14]), "=r"(d[15])
        : "r"(tmem + ((unsigned)(quarter * 32) << 16) + (unsigned)cb));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    const int row = row0 + quarter * 32 + lane;
    if (row < n) {
      float z[DC], h[DC];
#pragma unroll
      for (int e = 0; e < DC; ++e) {
        z[e] = __uint_as_float(d[e]) + bias[cb + e];
        h[e] = fmaxf(z[e], 0.f);
      }
      if (res) {  // res: KH == HID
        using IO = FeatIO<TIN>;
        const typename IO::Chunk* hin = reinterpret_cast<const typename IO::Chunk*>(Hin + (size_t)row * KH + cb);
#pragma unroll
        for (int c = 0; c < DC / IO::PER; ++c) {
          const typename IO::Chunk v = hin[c];
#pragma unroll
          for (int e = 0; e < IO::PER; ++e) h[c * IO::PER + e] = IO::get(v, e) + h[c * IO::PER + e];
        }
      }
      if (Z) {
        float4* zr = reinterpret_cast<float4*>(Z + (size_t)row * HID + cb);
#pragma unroll
        for (int c4 = 0; c4 < DC / 4; ++c4) zr[c4] = make_float4(z[4 * c4], z[4 * c4 + 1], z[4 * c4 + 2], z[4 * c4 + 3]);
      }
      store_feat(Hout + (size_t)row * HID + cb, h);
    }
    // every warp has read D and the tensor cores are done with A before the
    // next tile writes them
    tc_fence_before();
    __syncthreads();
  }
  tc_fence_after();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_COLS) : "memory");
}

// readout: gd_i = 1 + H_i . rd ; gl_k = what_k sum_c ro_c H_ic H_jc (j = col_k < i).
// Four lanes per row, eight features each: the 128-byte rows of H are read
// coalesced and the dot products finish with two shuffles.
constexpr int RO_LANES = 4;
constexpr int RO_F = HID / RO_LANES;
// the RO_F features of lane q's quarter of row i
template <typename T>
__device__ __forceinline__ void load_quarter(const T* __restrict__ H, int i, int q, float (&v)[RO_F]) {
  using IO = FeatIO<T>;
  const typename IO::Chunk* p = reinterpret_cast<const typename IO::Chunk*>(H + (size_t)i * HID + q * RO_F);
#pragma unroll
  for (int c = 0; c < RO_F / IO::PER; ++c) {
    const typename IO::Chunk ch = p[c];
#pragma unroll
    for (int e = 0; e < IO::PER; ++e) v[c * IO::PER + e] = IO::get(ch, e);
  }
}

template <typename T>
__global__ void k_readout(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                          const float* __restrict__ what, const T* __restrict__ H, const float* __restrict__ params,
                          float* gd, float* gl) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = gt / RO_LANES, q = gt % RO_LANES;
  const bool on = i < n;  // whole groups of four lanes share a row
  const float* rd = params + OFF_RD + q * RO_F;
  const float* ro = params + OFF_RO + q * RO_F;
  float hro[RO_F];
  float d = 0.f;
  if (on) {
    float hi[RO_F];
    load_quarter(H, i, q, hi);
#pragma unroll
    for (int c = 0; c < RO_F; ++c) {
      const float h = hi[c];
      d = fmaf(h, rd[c], d);
      hro[c] = h * ro[c];
    }
  }
  d += __shfl_xor_sync(0xffffffffu, d, 1);
  d += __shfl_xor_sync(0xffffffffu, d, 2);
  if (on && q == 0) gd[i] = 1.f + d;
  const int a = on ? rowptr[i] : 0, b = on ? rowptr[i + 1] : 0;
  // the four lanes of a row run the same trip count and shuffle among themselves
  const unsigned gmask = 0xFu << ((threadIdx.x & 31) & ~(RO_LANES - 1));
  for (int k = a; k < b; ++k) {
    const int j = col[k];
    float v = 0.f;
    if (j < i) {
      float hj[RO_F];
      load_quarter(H, j, q, hj);
#pragma unroll
      for (int c = 0; c < RO_F; ++c) v = fmaf(hro[c], hj[c], v);
    }
    v += __shfl_xor_sync(gmask, v, 1);
    v += __shfl_xor_sync(gmask, v, 2);
    if (q == 0) gl[k] = (j < i) ? v * what[k] : 0.f;
  }
}

// two-hop readout: gl2_e = pw_e sum_c ro2_c H_ic H_jc (j = col2_e < i), four lanes per row
template <typename T>
__global__ void k_readout2(int n, const int* __restrict__ rowptr2, const int* __restrict__ col2,
                           const float* __restrict__ pw, const T* __restrict__ H,
                           const float* __restrict__ params, float* gl2) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = gt / RO_LANES, q = gt % RO_LANES;
  const bool on = i < n;
  const float* ro2 = params + OFF_RO2 + q * RO_F;
  float hro[RO_F];
#pragma unroll
  for (int c = 0; c < RO_F; ++c) hro[c] = 0.f;
  if (on) {
    float hi[RO_F];
    load_quarter(H, i, q, hi);
#pragma unroll
    for (int c = 0; c < RO_F; ++c) hro[c] = hi[c] * ro2[c];
  }
  const int a = on ? rowptr2[i] : 0, b = on ? rowptr2[i + 1] : 0;
  const unsigned gmask = 0xFu << ((threadIdx.x & 31) & ~(RO_LANES - 1));
  for (int e = a; e < b; ++e) {
    const int j = col2[e];
    float v = 0.f;
    if (j < i) {
      float hj[RO_F];
      load_quarter(H, j, q, hj);
#pragma unroll
      for (int c = 0; c < RO_F; ++c) v = fmaf(hro[c], hj[c], v);
    }
    v += __shfl_xor_sync(gmask, v, 1);
    v += __shfl_xor_sync(gmask, v, 2);
    if (q == 0) gl2[e] = (j < i) ? v * pw[e] : 0.f;
  }
}

// ---------------------------------------------------------------- loss

__device__ __forceinline__ float probe_value(unsigned long long seed, int p, int i) {
  unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(p * 0x100000001ull + (unsigned)i + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (z & 1ull) ? 1.f : -1.f;
}

__global__ void k_probes(int n, int K, unsigned long long seed, float* Zp) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int p = 0; p < K; ++p) Zp[(size_t)p * n + i] = probe_value(seed, p, i);
}

// out = Gt^T in : out_i = gd_i in_i + sum_{k: col_k > i} gl[rev_k] in_col
__global__ void k_gt(int n, int K, const int* __restrict__ rowptr, const int* __restrict__ col,
                     const int* __restrict__ rev, const float* __restrict__ gd, const float* __restrict__ gl,
                     const float* __restrict__ in, float* out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int p = 0; p < K; ++p) {
    const float* v = in + (size_t)p * n;
    float acc = gd[i] * v[i];
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      const int j = col[k];
      if (j > i && rev[k] >= 0) acc = fmaf(gl[rev[k]], v[j], acc);
    }
    out[(size_t)p * n + i] = acc;
  }
}

// out = Gt in : out_i = gd_i in_i + sum_{k: col_k < i} gl_k in_col
__global__ void k_g(int n, int K, const int* __restrict__ rowptr, const int* __restrict__ col,
                    const float* __restrict__ gd, const float* __restrict__ gl, const float* __restrict__ in,
                    float* out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int p = 0; p < K; ++p) {
    const float* v = in + (size_t)p * n;
    float acc = gd[i] * v[i];
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      const int j = col[k];
      if (j < i) acc = fmaf(gl[k], v[j], acc);
    }
    out[(size_t)p * n + i] = acc;
  }
}

// out = At in = in - What in
__global__ void k_at(int n, int K, const int* __restrict__ rowptr, const int* __restrict__ col,
                     const float* __restrict__ what, const float* __restrict__ in, float* out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int p = 0; p < K; ++p) {
    const float* v = in + (size_t)p * n;
    float acc = v[i];
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) acc = fmaf(-what[k], v[col[k]], acc);
    out[(size_t)p * n + i] = acc;
  }
}

// r = u - z, block partial of sum r^2 (double)
__global__ void k_resid(int n, int K, const float* __restrict__ u, const float* __restrict__ z, float* r,
                        double* part) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    for (int p = 0; p < K; ++p) {
      const size_t o = (size_t)p * n + i;
      const float v = u[o] - z[o];
      r[o] = v;
      s += (double)v * (double)v;
    }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
    part[blockIdx.x] = t;
  }
}

// dGt entries: dgd_i = scale sum_p 2 (r_i t_i + z_i s_i); dgl_k = scale sum_p 2 (r_i t_j + z_i s_j), j < i
__global__ void k_gradG(int n, int K, const int* __restrict__ rowptr, const int* __restrict__ col,
                        const float* __restrict__ r, const float* __restrict__ t, const float* __restrict__ z,
                        const float* __restrict__ s, float scale, float* dgd, float* dgl) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float d = 0.f;
  for (int p = 0; p < K; ++p) {
    const size_t o = (size_t)p * n;
    d += 2.f * (r[o + i] * t[o + i] + z[o + i] * s[o + i]);
  }
  dgd[i] = scale * d;
  for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
    const int j = col[k];
    float v = 0.f;
    if (j < i)
      for (int p = 0; p < K; ++p) {
        const size_t o = (size_t)p * n;
        v += 2.f * (r[o + i] * t[o + j] + z[o + i] * s[o + j]);
      }
    dgl[k] = scale * v;
  }
}

// Exact FSAI (Kaporin) objective, one thread per row i with S_i = {i} and the
// lower neighbours of i (the pattern of row i of Gt):
//     L = (1/n) sum_i [ g_i^T At g_i - 2 log Gt_ii ],   g_i = row i of Gt,
// whose minimiser on the pattern is the FSAI factor (each row solves
// At[S,S] g = e_i / g_ii).  tv_j = (Gt At)_ij = g_j - sum_{m in S, m ~ j}
// g_m what(m, j) for j in S; dL/dGt_ij = (2 tv_j - [j = i] 2 / Gt_ii) / n.
constexpr int KMAX = 1 + LV_MAX_EDGES + Q2MAX;
__global__ void k_kaporin(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                          const float* __restrict__ what, const float* __restrict__ gd, const float* __restrict__ gl,
                          const int* __restrict__ rowptr2, const int* __restrict__ col2,
                          const float* __restrict__ gl2, float scale, float* dgd, float* dgl, float* dgl2,
                          double* part) {
  __shared__ double sh[32];
  double lsum = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int a = rowptr[i], b = rowptr[i + 1];
    // members of row i's pattern: i, its lower neighbours (kind 1) and its
    // lower two-hop neighbours (kind 2), with their entry positions
    int mem[KMAX], pos[KMAX], kind[KMAX];
    float g[KMAX], tv[KMAX];
    int S = 0;
    mem[S] = i;
    pos[S] = -1;
    kind[S] = 0;
    g[S] = gd[i];
    ++S;
    for (int k = a; k < b && S < KMAX; ++k)
      if (col[k] < i) {
        mem[S] = col[k];
        pos[S] = k;
        kind[S] = 1;
        g[S] = gl[k];
        ++S;
      }
    if (rowptr2)
      for (int e = rowptr2[i]; e < rowptr2[i + 1] && S < KMAX; ++e)
        if (col2[e] < i) {
          mem[S] = col2[e];
          pos[S] = e;
          kind[S] = 2;
          g[S] = gl2[e];
          ++S;
        }
    for (int p = 0; p < S; ++p) tv[p] = g[p];
    // tv_p -= g_q what(m_q -> m_p) for every member q and neighbour m_p of m_q
    for (int q = 0; q < S; ++q) {
      const int m = mem[q];
      for (int t = rowptr[m]; t < rowptr[m + 1]; ++t) {
        const int j = col[t];
        if (j > i) continue;  // members are <= i
        for (int p = 0; p < S; ++p)
          if (mem[p] == j) {
            tv[p] = fmaf(-g[q], what[t], tv[p]);
            break;
          }
      }
    }
    const float gii = fmaxf(g[0], 1e-6f);
    float li = -2.f * logf(gii);
    for (int p = 0; p < S; ++p) li = fmaf(g[p], tv[p], li);
    lsum += (double)li;
    dgd[i] = scale * (2.f * tv[0] - 2.f / gii);
    for (int k = a; k < b; ++k) dgl[k] = 0.f;
    if (rowptr2)
      for (int e = rowptr2[i]; e < rowptr2[i + 1]; ++e) dgl2[e] = 0.f;
    for (int p = 1; p < S; ++p) {
      if (kind[p] == 1) dgl[pos[p]] = scale * 2.f * tv[p];
      else dgl2[pos[p]] = scale * 2.f * tv[p];
    }
  }
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = lsum;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
    part[blockIdx.x] = t;
  }
}

// ---------------------------------------------------------------- backward

// dH_i from the readout; block partials of d rd, d ro and d ro2 (32 each)
__global__ void k_readout_bwd(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                              const int* __restrict__ rev, const float* __restrict__ what, const float* __restrict__ H,
                              const float* __restrict__ params, const float* __restrict__ dgd,
                              const float* __restrict__ dgl, const int* __restrict__ rowptr2,
                              const int* __restrict__ col2, const int* __restrict__ rev2,
                              const float* __restrict__ pw, const float* __restrict__ dgl2, float* dH, float* part) {
  // four lanes per row, a quarter of the features each (the forward readout's
  // layout): the 128-byte rows of H and dH move coalesced
  const int q = threadIdx.x % RO_LANES;
  const float* rd = params + OFF_RD + q * RO_F;
  const float* ro = params + OFF_RO + q * RO_F;
  const float* ro2 = params + OFF_RO2 + q * RO_F;
  float prd[RO_F], pro[RO_F], pro2[RO_F];
#pragma unroll
  for (int c = 0; c < RO_F; ++c) prd[c] = pro[c] = pro2[c] = 0.f;
  const int rows_per_round = gridDim.x * (blockDim.x / RO_LANES);
  for (int i = blockIdx.x * (blockDim.x / RO_LANES) + threadIdx.x / RO_LANES; i < n; i += rows_per_round) {
    float hi[RO_F], dh[RO_F];
    load_quarter(H, i, q, hi);
    const float gdi = dgd[i];
#pragma unroll
    for (int c = 0; c < RO_F; ++c) {
      dh[c] = gdi * rd[c];
      prd[c] = fmaf(gdi, hi[c], prd[c]);
    }
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      const int j = col[k];
      float coef;
      float hj[RO_F];
      load_quarter(H, j, q, hj);
      if (j < i) {
        coef = dgl[k] * what[k];
#pragma unroll
        for (int c = 0; c < RO_F; ++c) pro[c] = fmaf(coef * hi[c], hj[c], pro[c]);
      } else {
        const int rk = rev[k];
        coef = rk >= 0 ? dgl[rk] * what[rk] : 0.f;
      }
#pragma unroll
      for (int c = 0; c < RO_F; ++c) dh[c] = fmaf(coef * ro[c], hj[c], dh[c]);
    }
    if (rowptr2)
      for (int e = rowptr2[i]; e < rowptr2[i + 1]; ++e) {
        const int j = col2[e];
        float coef;
        float hj[RO_F];
        load_quarter(H, j, q, hj);
        if (j < i) {
          coef = dgl2[e] * pw[e];
#pragma unroll
          for (int c = 0; c < RO_F; ++c) pro2[c] = fmaf(coef * hi[c], hj[c], pro2[c]);
        } else {
          const int re = rev2[e];
          coef = re >= 0 ? dgl2[re] * pw[re] : 0.f;
        }
#pragma unroll
        for (int c = 0; c < RO_F; ++c) dh[c] = fmaf(coef * ro2[c], hj[c], dh[c]);
      }
    float4* o = reinterpret_cast<float4*>(dH + (size_t)i * HID + q * RO_F);
#pragma unroll
    for (int c4 = 0; c4 < RO_F / 4; ++c4) o[c4] = make_float4(dh[4 * c4], dh[4 * c4 + 1], dh[4 * c4 + 2], dh[4 * c4 + 3]);
  }
  // block reduction in a fixed order: the warp's rows (lanes of equal q),
  // then the warps in order
#pragma unroll
  for (int c = 0; c < RO_F; ++c) {
    float a = prd[c], b = pro[c], d = pro2[c];
    for (int off = 16; off >= RO_LANES; off >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, off);
      b += __shfl_down_sync(0xffffffffu, b, off);
      d += __shfl_down_sync(0xffffffffu, d, off);
    }
    prd[c] = a;
    pro[c] = b;
    pro2[c] = d;
  }
  __shared__ float swarp[8][3 * HID];
  if ((threadIdx.x & 31) < RO_LANES)
    for (int c = 0; c < RO_F; ++c) {
      swarp[threadIdx.x >> 5][q * RO_F + c] = prd[c];
      swarp[threadIdx.x >> 5][HID + q * RO_F + c] = pro[c];
      swarp[threadIdx.x >> 5][2 * HID + q * RO_F + c] = pro2[c];
    }
  __syncthreads();
  if (threadIdx.x < 3 * HID) {
    float t = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += swarp[w][threadIdx.x];
    part[(size_t)blockIdx.x * 3 * HID + threadIdx.x] = t;
  }
}

// Layer backward on tcgen05, 128-row tiles: dZ = dHout * [Z > 0];
// dXcat = dZ W^T into dHdir (first KH columns) and dAgg (last KH); the
// block's partials of dW = Xcat^T dZ and db = sum dZ.  Per tile two sets of
// products, issued by one thread and committed to one mbarrier:
//   dX: A = dZ (128 rows x 32, K-major), B = W as N x K (N = 2KH features,
//       K = 32 hidden: element (f, h) = W[f][h]), D = tensor-memory columns
//       [0, 2KH), read back by every warp after the tile;
//   dW: A = Xcat^T (M = 128: the 2KH features, then zero rows; K = the
//       tile's 128 rows), B = dZ^T as N x K (N = 32 hidden), D = columns
//       [BW_DW, BW_DW + 32), accumulated over all the block's tiles and read
//       once at the end (lane = feature).
// Operands are BF16 in the canonical no-swizzle K-major layout of the
// forward (umma_off); the transposed operands are written transposed.  The
// aggregation Agg(Hin) is the one the training forward stored, so the layer
// streams its rows instead of gathering neighbours.  Four blocks share an SM
// (53 KB of shared memory each, 4 x 128 = all 512 tensor-memory columns).
constexpr int BW_ROWS = 128;                 // rows of a tile (the K of the dW products)
constexpr unsigned BW_COLS = 128;            // tensor-memory columns: dX [0, 64), dW [64, 96)
constexpr unsigned BW_DW = 64;
constexpr int BW_XT = 0;                     // Xcat^T: 128 x 128 BF16
constexpr int BW_DZT = BW_XT + 128 * BW_ROWS * 2;   // dZ^T: 32 x 128
constexpr int BW_DZ = BW_DZT + HID * BW_ROWS * 2;   // dZ: 128 x 32
constexpr int BW_W = BW_DZ + BW_ROWS * HID * 2;     // W: 2KH x 32
constexpr size_t bwd_smem(int K) { return (size_t)BW_W + (size_t)K * HID * 2; }
__host__ __device__ constexpr unsigned tc_idesc(int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(N >> 3) << 17) | ((unsigned)(BW_ROWS >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(unsigned d, unsigned long long a, unsigned long long b, unsigned idesc,
                                       unsigned acc) {
  asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
                   d),
               "l"(a), "l"(b), "r"(idesc), "r"(acc)
               : "memory");
}
// 16 consecutive tensor-memory columns of the warp's 32 lanes (thread = lane)
__device__ __forceinline__ void tc_ld16(unsigned addr, float (&v)[16]) {
  uint32_t d[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]), "=r"(d[6]), "=r"(d[7]), "=r"(d[8]),
        "=r"(d[9]), "=r"(d[10]), "=r"(d[11]), "=r"(d[12]), "=r"(d[13]), "=r"(d[14]), "=r"(d[15])
      : "r"(addr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int e = 0; e < 16; ++e) v[e] = __uint_as_float(d[e]);
}

template <int KH>
__global__ void __launch_bounds__(TC_TPB, 4) k_layer_bwd(int n, const float* __restrict__ Hin,
                                                      const float* __restrict__ Agg,
                                                      const __nv_bfloat16* __restrict__ W, const float* __restrict__ Z,
                                                      const float* __restrict__ dHout, float* dHdir, float* dAgg,
                                                      float* partW, float* partb, int need_dx, int* status) {
  constexpr int K = 2 * KH, FH = KH / 2;
  static_assert(K % 16 == 0 && K <= 64, "2KH features in steps of 16, at most 64");
  extern __shared__ __align__(128) unsigned char bsm[];
  unsigned char* sXt = bsm + BW_XT;
  unsigned char* sDzt = bsm + BW_DZT;
  unsigned char* sDz = bsm + BW_DZ;
  unsigned char* sW = bsm + BW_W;
  __shared__ __align__(8) unsigned long long s_bar;
  __shared__ unsigned s_tmem;
  __shared__ float sB[TC_TPB / 32][HID];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned bar = (unsigned)__cvta_generic_to_shared(&s_bar);
  // W as N x K: element (f, h) = W[f * 32 + h]; Xcat^T's rows past K stay zero
  for (int t = threadIdx.x; t < K * HID; t += TC_TPB)
    *reinterpret_cast<__nv_bfloat16*>(sW + umma_off(t / HID, t % HID, HID)) = W[t];
  for (int t = threadIdx.x; t < 128 * BW_ROWS / 2; t += TC_TPB) reinterpret_cast<uint32_t*>(sXt)[t] = 0u;
  if (warp == 0) {
    const unsigned holder = (unsigned)__cvta_generic_to_shared(&s_tmem);
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(holder), "r"(BW_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = s_tmem;
  const unsigned long long xt_desc = umma_desc(sXt, 128, BW_ROWS * 16);
  const unsigned long long dzt_desc = umma_desc(sDzt, 128, BW_ROWS * 16);
  const unsigned long long dz_desc = umma_desc(sDz, 128, HID * 16);
  const unsigned long long w_desc = umma_desc(sW, 128, HID * 16);
  const int ntiles = (n + BW_ROWS - 1) / BW_ROWS;
  const int rl = warp * 16;  // the warp's 16 rows of the tile
  unsigned parity = 0;
  bool ok = true, any = false;
  float accB = 0.f;  // lane = column of db
  for (int tl = blockIdx.x; tl < ntiles && ok; tl += gridDim.x) {
    const int row0 = tl * BW_ROWS;
    {
      // Xcat^T: lane (r, half) writes its row's features as column rl + r;
      // the aggregation is the forward's (Agg), rows past n are zeros
      const int r = lane & 15, half = lane >> 4;
      const int row = row0 + rl + r;
      float own[FH], agg[FH];
#pragma unroll
      for (int f = 0; f < FH; ++f) own[f] = agg[f] = 0.f;
      if (row < n) {
        const float4* ho = reinterpret_cast<const float4*>(Hin + (size_t)row * KH + half * FH);
        const float4* ha = reinterpret_cast<const float4*>(Agg + (size_t)row * KH + half * FH);
#pragma unroll
        for (int c4 = 0; c4 < FH / 4; ++c4) {
          const float4 a = ho[c4], b = ha[c4];
          own[4 * c4] = a.x; own[4 * c4 + 1] = a.y; own[4 * c4 + 2] = a.z; own[4 * c4 + 3] = a.w;
          agg[4 * c4] = b.x; agg[4 * c4 + 1] = b.y; agg[4 * c4 + 2] = b.z; agg[4 * c4 + 3] = b.w;
        }
      }
#pragma unroll
      for (int f = 0; f < FH; ++f) {
        *reinterpret_cast<__nv_bfloat16*>(sXt + umma_off(half * FH + f, rl + r, BW_ROWS)) = __float2bfloat16_rn(own[f]);
        *reinterpret_cast<__nv_bfloat16*>(sXt + umma_off(KH + half * FH + f, rl + r, BW_ROWS)) =
            __float2bfloat16_rn(agg[f]);
      }
    }
    // dZ and dZ^T: lane = hidden column, over the warp's 16 rows
#pragma unroll 4
    for (int r = 0; r < 16; ++r) {
      const int row = row0 + rl + r;
      float v = 0.f;
      if (row < n) {
        const size_t o = (size_t)row * HID + lane;
        v = Z[o] > 0.f ? dHout[o] : 0.f;
      }
      accB += v;
      const __nv_bfloat16 b = __float2bfloat16_rn(v);
      *reinterpret_cast<__nv_bfloat16*>(sDz + umma_off(rl + r, lane, HID)) = b;
      *reinterpret_cast<__nv_bfloat16*>(sDzt + umma_off(lane, rl + r, BW_ROWS)) = b;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the operands, for the tensor cores
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0) {
      tc_fence_after();
      if (need_dx) {
#pragma unroll
        for (int ks = 0; ks < HID / 16; ++ks)
          tc_mma(tmem, dz_desc + (unsigned long long)ks * 16, w_desc + (unsigned long long)ks * 16, tc_idesc(K),
                 ks > 0 ? 1u : 0u);
      }
#pragma unroll
      for (int ks = 0; ks < BW_ROWS / 16; ++ks)
        tc_mma(tmem + BW_DW, xt_desc + (unsigned long long)ks * 16, dzt_desc + (unsigned long long)ks * 16,
               tc_idesc(HID), (any || ks > 0) ? 1u : 0u);
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                   : "memory");
    }
    any = true;
    // bounded wait; on a timeout a second bounded wait lets the products in
    // flight finish before the block gives up
    const bool done = tc_bar_wait(bar, parity);
    if (!__syncthreads_and(done)) {
      if (threadIdx.x == 0) atomicOr(status, LV_FLAG_BARRIER_TIMEOUT);
      tc_bar_wait(bar, parity);
      ok = false;
      break;
    }
    parity ^= 1u;
    tc_fence_after();
    if (need_dx) {
      // warp w: lanes 32 (w % 4) .. + 31 (rows), columns (w / 4) K/2 .. + K/2 - 1
      const int quarter = warp & 3, cb = (warp >> 2) * (K / 2);
      const int row = row0 + quarter * 32 + lane;
#pragma unroll
      for (int c0 = 0; c0 < K / 2; c0 += 16) {
        float v[16];
        tc_ld16(tmem + ((unsigned)(quarter * 32) << 16) + (unsigned)(cb + c0), v);
        if (row < n) {
          const int c = cb + c0;  // 16 columns on one side of KH (KH is a multiple of 16)
          float* dst = c < KH ? dHdir + (size_t)row * KH + c : dAgg + (size_t)row * KH + (c - KH);
          float4* d4 = reinterpret_cast<float4*>(dst);
#pragma unroll
          for (int q = 0; q < 4; ++q) d4[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        }
      }
    }
    // every warp has read dX and the tensor cores are done with the operands
    // before the next tile writes them
    tc_fence_before();
    __syncthreads();
  }
  tc_fence_after();
  // dW: warp w reads features 32 (w % 4) + lane, hidden columns 16 (w / 4) .. + 15
  {
    const int quarter = warp & 3, hb = (warp >> 2) * 16;
    const int f = quarter * 32 + lane;
    float v[16];
    if (any && ok) {
      tc_ld16(tmem + ((unsigned)(quarter * 32) << 16) + BW_DW + (unsigned)hb, v);
    } else {
#pragma unroll
      for (int e = 0; e < 16; ++e) v[e] = 0.f;
    }
    if (f < K) {
      float4* d4 = reinterpret_cast<float4*>(partW + (size_t)blockIdx.x * K * HID + (size_t)f * HID + hb);
#pragma unroll
      for (int q = 0; q < 4; ++q) d4[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    }
  }
  sB[warp][lane] = accB;
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x < HID) {
    float t = 0.f;
    for (int w = 0; w < TC_TPB / 32; ++w) t += sB[w][threadIdx.x];
    partb[(size_t)blockIdx.x * HID + threadIdx.x] = t;
  }
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BW_COLS) : "memory");
}

// dHin_j = dHdir_j + (res ? dHout_j : 0) + sum_{i ~ j} what_ij dAgg_i, four
// lanes per row (a quarter of the 32 features each, the rows coalesced), two
// neighbours' loads per round; every feature sums in the same order as one
// thread per row would.
__global__ void k_agg_bwd(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                          const int* __restrict__ rev, const float* __restrict__ what,
                          const float* __restrict__ dHdir, const float* __restrict__ dAgg,
                          const float* __restrict__ dHout, int res, float* dHin) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = gt / RO_LANES, q = gt % RO_LANES;
  if (j >= n) return;
  float acc[RO_F];
  load_quarter(dHdir, j, q, acc);
  if (res) {
    float h[RO_F];
    load_quarter(dHout, j, q, h);
#pragma unroll
    for (int f = 0; f < RO_F; ++f) acc[f] = acc[f] + h[f];
  }
  const int k1 = rowptr[j + 1];
  for (int k = rowptr[j]; k < k1; k += 2) {
    const bool two = k + 1 < k1;
    const int r0 = rev[k], r1 = two ? rev[k + 1] : -1;
    const int i0 = col[k], i1 = two ? col[k + 1] : i0;
    const float w0 = r0 >= 0 ? what[r0] : 0.f, w1 = r1 >= 0 ? what[r1] : 0.f;
    float d0[RO_F], d1[RO_F];
    load_quarter(dAgg, i0, q, d0);
    load_quarter(dAgg, i1, q, d1);
    if (r0 >= 0) {
#pragma unroll
      for (int f = 0; f < RO_F; ++f) acc[f] = fmaf(w0, d0[f], acc[f]);
    }
    if (r1 >= 0) {
#pragma unroll
      for (int f = 0; f < RO_F; ++f) acc[f] = fmaf(w1, d1[f], acc[f]);
    }
  }
  float4* o = reinterpret_cast<float4*>(dHin + (size_t)j * HID + q * RO_F);
#pragma unroll
  for (int c4 = 0; c4 < RO_F / 4; ++c4) o[c4] = make_float4(acc[4 * c4], acc[4 * c4 + 1], acc[4 * c4 + 2], acc[4 * c4 + 3]);
}

// sum block partials (fixed order) into grad[off..off+len)
__global__ void k_sum_parts(const float* __restrict__ part, int nblocks, int len, float* grad) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= len) return;
  float s = 0.f;
  for (int b = 0; b < nblocks; ++b) s += part[(size_t)b * len + t];
  grad[t] = s;
}

__global__ void k_sum_loss(const double* part, int nb, double scale, double* out) {
  if (threadIdx.x != 0) return;
  double s = 0.0;
  for (int b = 0; b < nb; ++b) s += part[b];
  out[0] = s * scale;
}

__global__ void k_adam(int np, float* p, const float* __restrict__ gr, float* m1, float* m2, float lr, float b1,
                       float b2, float c1, float c2) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const float gi = gr[i];
  const float a = b1 * m1[i] + (1.f - b1) * gi;
  const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
  m1[i] = a;
  m2[i] = b;
  p[i] -= lr * (a / c1) / (sqrtf(b / c2) + 1e-8f);
}

__global__ void k_to_bf16(const float* __restrict__ p, __nv_bfloat16* wbf) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < KC0 * HID) wbf[WBF_W0 + t] = __float2bfloat16_rn(p[OFF_W0 + t]);
  if (t < KC * HID) {
    wbf[WBF_W1 + t] = __float2bfloat16_rn(p[OFF_W1 + t]);
    wbf[WBF_W2 + t] = __float2bfloat16_rn(p[OFF_W2 + t]);
  }
}

}  // namespace

// ======================================================================= host

struct LearnSystem {
  int n = 0;
  int nnz = 0;
  int* rowptr = nullptr;
  int* col = nullptr;
  double* w = nullptr;
  double* diag = nullptr;
  double* adiag = nullptr;
};

struct LearnState {
  float *params = nullptr, *grad = nullptr, *m1 = nullptr, *m2 = nullptr;
  __nv_bfloat16* wbf = nullptr;
  bool wbf_valid = false;  // wbf holds the current weights (set by every forward that converts them)
  int adam_t = 0;
  int cap = 0;
  int64_t nnz_cap = 0;
  // workspace
  float *dh, *what, *X, *H1, *H2, *H3, *Z0, *Z1, *Z2, *gd, *gl;
  int* rev;
  float *dH3, *dH2, *dH1, *dHdir, *dAgg, *dgd, *dgl;
  float *zp, *y, *t, *u, *r, *v, *s;
  float *partW, *partb, *partR;
  double *partL, *loss;
  // training: each layer's aggregation Agg(Hin), kept by the forward for the
  // backward (allocated by the first training forward)
  float *A0 = nullptr, *A1 = nullptr, *A2 = nullptr;
  // two-hop pattern (hops == 2), built per system in prepare()
  int hops = 1;
  int *rowptr2 = nullptr, *col2 = nullptr, *rev2 = nullptr, *q_overflow = nullptr;
  float *pw = nullptr, *gl2 = nullptr, *dgl2 = nullptr;
  std::vector<LearnSystem> systems;
  std::vector<void*> allocs;
  bool factor_ready = false;
};

namespace {

template <class T>
T* lalloc(LearnState* L, size_t count) {
  void* p = nullptr;
  if (count == 0) count = 1;
  if (cudaMalloc(&p, sizeof(T) * count) != cudaSuccess) return nullptr;
  cudaMemset(p, 0, sizeof(T) * count);
  L->allocs.push_back(p);
  return static_cast<T*>(p);
}

unsigned long long splitmix(unsigned long long& s) {
  unsigned long long z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

float gauss(unsigned long long& s) {
  const double u1 = ((splitmix(s) >> 11) + 1.0) * (1.0 / 9007199254740993.0);
  const double u2 = (splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
  return (float)(sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2));
}

int ensure_state(lv_ctx* c) {
  if (c->learn) return LV_OK;
  LearnState* L = new LearnState();
  L->cap = c->cap;
  L->nnz_cap = c->sv.nnz_cap;
  const size_t cap = c->cap, nnz = (size_t)c->sv.nnz_cap;
  L->params = lalloc<float>(L, NPARAM);
  L->grad = lalloc<float>(L, NPARAM);
  L->m1 = lalloc<float>(L, NPARAM);
  L->m2 = lalloc<float>(L, NPARAM);
  L->wbf = lalloc<__nv_bfloat16>(L, NWBF);
  L->dh = lalloc<float>(L, cap);
  L->what = lalloc<float>(L, nnz);
  L->rev = lalloc<int>(L, nnz);
  L->X = lalloc<float>(L, cap * FIN);
  for (float** p : {&L->H1, &L->H2, &L->H3, &L->Z0, &L->Z1, &L->Z2, &L->dH3, &L->dH2, &L->dH1, &L->dHdir, &L->dAgg})
    *p = lalloc<float>(L, cap * HID);
  L->gd = lalloc<float>(L, cap);
  L->gl = lalloc<float>(L, nnz);
  L->dgd = lalloc<float>(L, cap);
  L->dgl = lalloc<float>(L, nnz);
  for (float** p : {&L->zp, &L->y, &L->t, &L->u, &L->r, &L->v, &L->s}) *p = lalloc<float>(L, cap * MAXPROBES);
  L->partW = lalloc<float>(L, (size_t)BW_BLOCKS * KC * HID);
  L->partb = lalloc<float>(L, (size_t)BW_BLOCKS * HID);
  L->partR = lalloc<float>(L, (size_t)RB_BLOCKS * 3 * HID);
  L->partL = lalloc<double>(L, PART_BLOCKS);
  L->loss = lalloc<double>(L, 4);
  bool ok = L->params && L->loss && L->partR && L->s;
  if (!ok) {
    for (void* p : L->allocs) cudaFree(p);
    delete L;
    return lv_fail(c, LV_ERR_CUDA, "learned preconditioner: out of device memory");
  }
  c->learn = L;
  return LV_OK;
}

int ensure_hop2(lv_ctx* c) {
  LearnState* L = c->learn;
  if (L->rowptr2) return LV_OK;
  const size_t cap = L->cap, q = (size_t)Q2MAX * L->cap;
  L->rowptr2 = lalloc<int>(L, cap + 1);
  L->col2 = lalloc<int>(L, q);
  L->rev2 = lalloc<int>(L, q);
  L->q_overflow = lalloc<int>(L, 1);
  L->pw = lalloc<float>(L, q);
  L->gl2 = lalloc<float>(L, q);
  L->dgl2 = lalloc<float>(L, q);
  if (!L->dgl2) return lv_fail(c, LV_ERR_CUDA, "learned preconditioner: out of device memory (two-hop pattern)");
  return LV_OK;
}

void init_params(LearnState* L, unsigned long long seed, cudaStream_t s) {
  std::vector<float> p(NPARAM, 0.f);
  unsigned long long st = seed ^ 0xA5A5A5A5ull;
  auto fill = [&](int off, int fan_in, int count, float gain) {
    const float sd = gain / sqrtf((float)fan_in);
    for (int k = 0; k < count; ++k) p[off + k] = sd * gauss(st);
  };
  fill(OFF_W0, KC0, KC0 * HID, 1.0f);
  fill(OFF_W1, KC, KC * HID, 0.5f);
  fill(OFF_W2, KC, KC * HID, 0.5f);
  fill(OFF_RD, HID, HID, 0.01f);
  fill(OFF_RO, HID, HID, 0.01f);
  fill(OFF_RO2, HID, HID, 0.01f);
  cudaMemcpyAsync(L->params, p.data(), sizeof(float) * NPARAM, cudaMemcpyHostToDevice, s);
  L->wbf_valid = false;
  cudaMemsetAsync(L->m1, 0, sizeof(float) * NPARAM, s);
  cudaMemsetAsync(L->m2, 0, sizeof(float) * NPARAM, s);
  L->adam_t = 0;
}

constexpr int TPB = 256;

// Features and normalised weights of one system.
int prepare(lv_ctx* c, const LearnSystem& S) {
  LearnState* L = c->learn;
  cudaStream_t s = c->stream;
  k_lprep_dh<<<lv_blocks(S.n, TPB), TPB, 0, s>>>(S.n, S.adiag, L->dh);
  k_lprep<<<lv_blocks(S.n, TPB), TPB, 0, s>>>(S.n, S.rowptr, S.col, S.w, S.diag, S.adiag, L->dh, L->what, L->rev, L->X);
  c->launches += 2;
  if (L->hops == 2) {
    if (int rc = ensure_hop2(c)) return rc;
    int* cnt = reinterpret_cast<int*>(L->dgl2);  // scratch for the counts
    k_hop2_count<<<lv_blocks(S.n, TPB), TPB, 0, s>>>(S.n, S.rowptr, S.col, L->what, cnt, L->q_overflow);
    if (int rc = lv_scan_int(c, cnt, L->rowptr2, S.n)) return rc;
    k_hop2_fill<<<lv_blocks(S.n, TPB), TPB, 0, s>>>(S.n, S.rowptr, S.col, L->what, L->rowptr2, L->col2, L->pw);
    k_hop2_rev<<<lv_blocks(S.n, TPB), TPB, 0, s>>>(S.n, L->rowptr2, L->col2, L->rev2);
    c->launches += 3;
  }
  return lv_cuda_check(c, cudaGetLastError(), "learned: prepare");
}

// infer: the per-step factor, which needs no pre-activations (Z is kept for
// the backward pass of training only)
int forward(lv_ctx* c, const LearnSystem& S, bool infer = false) {
  LearnState* L = c->learn;
  cudaStream_t s = c->stream;
  // 128-row tiles, all at once while they fit four blocks per SM (the
  // aggregation is latency-bound), else a persistent loop over the tiles
  const int nb = std::max(1, std::min((S.n + TC_ROWS - 1) / TC_ROWS, 4 * c->num_sms));
  if (!L->wbf_valid) {  // BF16 weights once per change of the parameters
    k_to_bf16<<<lv_blocks(KC * HID, TPB), TPB, 0, s>>>(L->params, L->wbf);
    L->wbf_valid = true;
    c->launches++;
  }
  const int gb = lv_blocks(S.n * RO_LANES, TPB);
  if (infer) {
    // the hidden features in BF16 (the buffers of the FP32 ones), no Z
    typedef __nv_bfloat16 B16;
    B16 *h1 = reinterpret_cast<B16*>(L->H1), *h2 = reinterpret_cast<B16*>(L->H2), *h3 = reinterpret_cast<B16*>(L->H3);
    k_layer_fwd<FIN, float, B16><<<nb, TC_TPB, 0, s>>>(S.n, L->X, S.rowptr, S.col, L->what, L->wbf + WBF_W0,
                                                         L->params + OFF_B0, 0, nullptr, h1, nullptr, c->status);
    k_layer_fwd<HID, B16, B16><<<nb, TC_TPB, 0, s>>>(S.n, h1, S.rowptr, S.col, L->what, L->wbf + WBF_W1,
                                                       L->params + OFF_B1, 1, nullptr, h2, nullptr, c->status);
    k_layer_fwd<HID, B16, B16><<<nb, TC_TPB, 0, s>>>(S.n, h2, S.rowptr, S.col, L->what, L->wbf + WBF_W2,
                                                       L->params + OFF_B2, 1, nullptr, h3, nullptr, c->status);
    k_readout<B16><<<gb, TPB, 0, s>>>(S.n, S.rowptr, S.col, L->what, h3, L->params, L->gd, L->gl);
    if (L->hops == 2) {
      k_readout2<B16><<<gb, TPB, 0, s>>>(S.n, L->rowptr2, L->col2, L->pw, h3, L->params, L->gl2);
      c->launches++;
    }
  } else {
    if (!L->A0) {
      L->A0 = lalloc<float>(L, (size_t)L->cap * FIN);
      L->A1 = lalloc<float>(L, (size_t)L->cap * HID);
      L->A2 = lalloc<float>(L, (size_t)L->cap * HID);
      if (!L->A0 || !L->A1 || !L->A2) return lv_fail(c, LV_ERR_CUDA, "learned: allocation of the training aggregations failed");
    }
    k_layer_fwd<FIN, float, float><<<nb, TC_TPB, 0, s>>>(S.n, L->X, S.rowptr, S.col, L->what, L->wbf + WBF_W0,
                                                           L->params + OFF_B0, 0, L->Z0, L->H1, L->A0, c->status);
    k_layer_fwd<HID, float, float><<<nb, TC_TPB, 0, s>>>(S.n, L->H1, S.rowptr, S.col, L->what, L->wbf + WBF_W1,
                                                           L->params + OFF_B1, 1, L->Z1, L->H2, L->A1, c->status);
    k_layer_fwd<HID, float, float><<<nb, TC_TPB, 0, s>>>(S.n, L->H2, S.rowptr, S.col, L->what, L->wbf + WBF_W2,
                                                           L->params + OFF_B2, 1, L->Z2, L->H3, L->A2, c->status);
    k_readout<float><<<gb, TPB, 0, s>>>(S.n, S.rowptr, S.col, L->what, L->H3, L->params, L->gd, L->gl);
    if (L->hops == 2) {
      k_readout2<float><<<gb, TPB, 0, s>>>(S.n, L->rowptr2, L->col2, L->pw, L->H3, L->params, L->gl2);
      c->launches++;
    }
  }
  c->launches += 4;
  return lv_cuda_check(c, cudaGetLastError(), "learned: forward");
}

// loss (into L->loss[0]) and dGt (L->dgd, L->dgl): the Hutchinson estimate
// with K probes in L->zp, or the exact FSAI (Kaporin) objective for K = 0
int loss_grad_G(lv_ctx* c, const LearnSystem& S, int K) {
  LearnState* L = c->learn;
  cudaStream_t s = c->stream;
  const int n = S.n, b = lv_blocks(n, TPB);
  if (K == 0) {
    const int nbl = std::min(PART_BLOCKS, b);
    const bool h2 = L->hops == 2;
    k_kaporin<<<nbl, TPB, 0, s>>>(n, S.rowptr, S.col, L->what, L->gd, L->gl, h2 ? L->rowptr2 : nullptr,
                                  h2 ? L->col2 : nullptr, h2 ? L->gl2 : nullptr, 1.0f / (float)n, L->dgd, L->dgl,
                                  h2 ? L->dgl2 : nullptr, L->partL);
    k_sum_loss<<<1, 32, 0, s>>>(L->partL, nbl, 1.0 / (double)n, L->loss);
    c->launches += 2;
    return lv_cuda_check(c, cudaGetLastError(), "learned: Kaporin loss");
  }
  k_gt<<<b, TPB, 0, s>>>(n, K, S.rowptr, S.col, L->rev, L->gd, L->gl, L->zp, L->y);
  k_at<<<b, TPB, 0, s>>>(n, K, S.rowptr, S.col, L->what, L->y, L->t);
  k_g<<<b, TPB, 0, s>>>(n, K, S.rowptr, S.col, L->gd, L->gl, L->t, L->u);
  const int nbl = std::min(PART_BLOCKS, b);
  k_resid<<<nbl, TPB, 0, s>>>(n, K, L->u, L->zp, L->r, L->partL);
  k_sum_loss<<<1, 32, 0, s>>>(L->partL, nbl, 1.0 / ((double)K * n), L->loss);
  k_gt<<<b, TPB, 0, s>>>(n, K, S.rowptr, S.col, L->rev, L->gd, L->gl, L->r, L->v);
  k_at<<<b, TPB, 0, s>>>(n, K, S.rowptr, S.col, L->what, L->v, L->s);
  k_gradG<<<b, TPB, 0, s>>>(n, K, S.rowptr, S.col, L->r, L->t, L->zp, L->s, 1.0f / ((float)K * n), L->dgd, L->dgl);
  c->launches += 8;
  return lv_cuda_check(c, cudaGetLastError(), "learned: loss");
}

int backward(lv_ctx* c, const LearnSystem& S) {
  LearnState* L = c->learn;
  cudaStream_t s = c->stream;
  const int n = S.n;
  const int nbr = std::min(RB_BLOCKS, lv_blocks(n * RO_LANES, TPB));
  const bool h2 = L->hops == 2;
  k_readout_bwd<<<nbr, TPB, 0, s>>>(n, S.rowptr, S.col, L->rev, L->what, L->H3, L->params, L->dgd, L->dgl,
                                    h2 ? L->rowptr2 : nullptr, h2 ? L->col2 : nullptr, h2 ? L->rev2 : nullptr,
                                    h2 ? L->pw : nullptr, h2 ? L->dgl2 : nullptr, L->dH3, L->partR);
  k_sum_parts<<<1, 3 * HID, 0, s>>>(L->partR, nbr, 3 * HID, L->grad + OFF_RD);
  const int nb = std::max(1, std::min(BW_BLOCKS, (n + BW_ROWS - 1) / BW_ROWS));
  // layer 2: Hin = H2, dHout = dH3
  k_layer_bwd<HID><<<nb, TC_TPB, bwd_smem(KC), s>>>(n, L->H2, L->A2, L->wbf + WBF_W2, L->Z2,
                                                     L->dH3, L->dHdir, L->dAgg, L->partW, L->partb, 1, c->status);
  k_sum_parts<<<lv_blocks(KC * HID, TPB), TPB, 0, s>>>(L->partW, nb, KC * HID, L->grad + OFF_W2);
  k_sum_parts<<<1, HID, 0, s>>>(L->partb, nb, HID, L->grad + OFF_B2);
  k_agg_bwd<<<lv_blocks(n * RO_LANES, TPB), TPB, 0, s>>>(n, S.rowptr, S.col, L->rev, L->what, L->dHdir, L->dAgg, L->dH3, 1,
                                                    L->dH2);
  // layer 1: Hin = H1, dHout = dH2
  k_layer_bwd<HID><<<nb, TC_TPB, bwd_smem(KC), s>>>(n, L->H1, L->A1, L->wbf + WBF_W1, L->Z1,
                                                     L->dH2, L->dHdir, L->dAgg, L->partW, L->partb, 1, c->status);
  k_sum_parts<<<lv_blocks(KC * HID, TPB), TPB, 0, s>>>(L->partW, nb, KC * HID, L->grad + OFF_W1);
  k_sum_parts<<<1, HID, 0, s>>>(L->partb, nb, HID, L->grad + OFF_B1);
  k_agg_bwd<<<lv_blocks(n * RO_LANES, TPB), TPB, 0, s>>>(n, S.rowptr, S.col, L->rev, L->what, L->dHdir, L->dAgg, L->dH2, 1,
                                                    L->dH1);
  // layer 0: Hin = X (no dX needed)
  k_layer_bwd<FIN><<<nb, TC_TPB, bwd_smem(KC0), s>>>(n, L->X, L->A0, L->wbf + WBF_W0, L->Z0,
                                                      L->dH1, L->dHdir, L->dAgg, L->partW, L->partb, 0, c->status);
  k_sum_parts<<<lv_blocks(KC0 * HID, TPB), TPB, 0, s>>>(L->partW, nb, KC0 * HID, L->grad + OFF_W0);
  k_sum_parts<<<1, HID, 0, s>>>(L->partb, nb, HID, L->grad + OFF_B0);
  c->launches += 14;
  return lv_cuda_check(c, cudaGetLastError(), "learned: backward");
}

LearnSystem current_system(lv_ctx* c) {
  LearnSystem S;
  S.n = c->n;
  S.rowptr = c->sv.rowptr;
  S.col = c->sv.col;
  S.w = c->sv.w;
  S.diag = c->sv.diag;
  S.adiag = c->sv.adiag;
  return S;
}

}  // namespace

// The backward layers' dynamic shared memory (above the 48 KB default) on the
// current device.
int lv_learn_device_setup() {
  cudaError_t e = cudaFuncSetAttribute(k_layer_bwd<HID>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bwd_smem(KC));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_layer_bwd<FIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bwd_smem(KC0));
  return e == cudaSuccess ? LV_OK : LV_ERR_CUDA;
}

// Inference for the currently assembled operator: fills gd, gl, dh, rev for
// the learned solve.  Called by the solver when the method is learned.
int lv_learn_factor_current(lv_ctx* c) {
  if (int rc = ensure_state(c)) return rc;
  // an untrained network (all parameters zero) gives Gt = I, i.e. Jacobi
  LearnSystem S = current_system(c);
  if (int rc = prepare(c, S)) return rc;
  return forward(c, S, true);
}

void lv_learn_free(lv_ctx* c) {
  if (!c->learn) return;
  for (void* p : c->learn->allocs) cudaFree(p);
  for (auto& S : c->learn->systems) {
    cudaFree(S.rowptr);
    cudaFree(S.col);
    cudaFree(S.w);
    cudaFree(S.diag);
    cudaFree(S.adiag);
  }
  delete c->learn;
  c->learn = nullptr;
}

void lv_learn_factor_ptrs(lv_ctx* c, const float** gd, const float** gl, const float** dh, const int** rev) {
  LearnState* L = c->learn;
  *gd = L ? L->gd : nullptr;
  *gl = L ? L->gl : nullptr;
  *dh = L ? L->dh : nullptr;
  *rev = L ? L->rev : nullptr;
}

void lv_learn_factor2_ptrs(lv_ctx* c, const int** rowptr2, const int** col2, const float** gl2, const int** rev2) {
  LearnState* L = c->learn;
  const bool h2 = L && L->hops == 2 && L->rowptr2;
  *rowptr2 = h2 ? L->rowptr2 : nullptr;
  *col2 = h2 ? L->col2 : nullptr;
  *gl2 = h2 ? L->gl2 : nullptr;
  *rev2 = h2 ? L->rev2 : nullptr;
}

extern "C" {

int lv_learn_init(lv_ctx* c, uint64_t seed) {
  if (c) c->factor_valid = false;
  if (!c) return LV_ERR_BAD_ARGUMENT;
  if (int rc = ensure_state(c)) return rc;
  init_params(c->learn, seed, c->stream);
  c->learn->factor_ready = true;
  return lv_cuda_check(c, cudaStreamSynchronize(c->stream), "lv_learn_init");
}

int32_t lv_learn_num_params(void) { return NPARAM; }

int lv_learn_get_params(lv_ctx* c, float* out) {
  if (!c || !out) return LV_ERR_BAD_ARGUMENT;
  if (int rc = ensure_state(c)) return rc;
  cudaMemcpyAsync(out, c->learn->params, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, c->stream);
  return lv_cuda_check(c, cudaStreamSynchronize(c->stream), "lv_learn_get_params");
}

int lv_learn_set_params(lv_ctx* c, const float* in) {
  if (c) c->factor_valid = false;
  if (!c || !in) return LV_ERR_BAD_ARGUMENT;
  if (int rc = ensure_state(c)) return rc;
  cudaMemcpyAsync(c->learn->params, in, sizeof(float) * NPARAM, cudaMemcpyHostToDevice, c->stream);
  c->learn->wbf_valid = false;
  c->learn->factor_ready = true;
  return lv_cuda_check(c, cudaStreamSynchronize(c->stream), "lv_learn_set_params");
}

int lv_learn_add_system(lv_ctx* c) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  if (!c->op_ready) return lv_fail(c, LV_ERR_NOT_MESHED, "the pressure operator has not been assembled");
  if (int rc = ensure_state(c)) return rc;
  LearnSystem S;
  S.n = c->n;
  int nnz = 0;
  cudaMemcpyAsync(&nnz, c->sv.rowptr + c->n, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return lv_cuda_check(c, e, "lv_learn_add_system");
  S.nnz = nnz;
  if (cudaMalloc(&S.rowptr, sizeof(int) * (S.n + 1)) != cudaSuccess || cudaMalloc(&S.col, sizeof(int) * nnz) ||
      cudaMalloc(&S.w, sizeof(double) * nnz) || cudaMalloc(&S.diag, sizeof(double) * S.n) ||
      cudaMalloc(&S.adiag, sizeof(double) * S.n))
    return lv_fail(c, LV_ERR_CUDA, "lv_learn_add_system: out of device memory");
  cudaMemcpyAsync(S.rowptr, c->sv.rowptr, sizeof(int) * (S.n + 1), cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(S.col, c->sv.col, sizeof(int) * nnz, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(S.w, c->sv.w, sizeof(double) * nnz, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(S.diag, c->sv.diag, sizeof(double) * S.n, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(S.adiag, c->sv.adiag, sizeof(double) * S.n, cudaMemcpyDeviceToDevice, c->stream);
  c->learn->systems.push_back(S);
  e = cudaStreamSynchronize(c->stream);
  return lv_cuda_check(c, e, "lv_learn_add_system");
}

int32_t lv_learn_num_systems(lv_ctx* c) { return (c && c->learn) ? (int32_t)c->learn->systems.size() : 0; }

int lv_learn_clear_systems(lv_ctx* c) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  if (!c->learn) return LV_OK;
  cudaStreamSynchronize(c->stream);
  for (auto& S : c->learn->systems) {
    cudaFree(S.rowptr);
    cudaFree(S.col);
    cudaFree(S.w);
    cudaFree(S.diag);
    cudaFree(S.adiag);
  }
  c->learn->systems.clear();
  return LV_OK;
}

// Loss and gradient on training system `sys` (or the current operator when
// sys < 0) for K probes (given as K x n floats, or Rademacher from `seed`
// when probes is NULL).  grad may be NULL.
int lv_learn_loss_grad(lv_ctx* c, int32_t sys, const float* probes, int32_t K, uint64_t seed, double* loss,
                       float* grad) {
  if (!c || K < 0 || K > MAXPROBES) return LV_ERR_BAD_ARGUMENT;
  if (int rc = ensure_state(c)) return rc;
  LearnState* L = c->learn;
  if (K > 0 && L->hops == 2)
    return lv_fail(c, LV_ERR_BAD_ARGUMENT, "the Hutchinson objective supports the one-hop pattern only");
  LearnSystem S;
  if (sys < 0) {
    if (!c->op_ready) return lv_fail(c, LV_ERR_NOT_MESHED, "the pressure operator has not been assembled");
    S = current_system(c);
  } else {
    if (sys >= (int)L->systems.size()) return LV_ERR_BAD_ARGUMENT;
    S = L->systems[sys];
  }
  cudaStream_t s = c->stream;
  if (int rc = prepare(c, S)) return rc;
  if (int rc = forward(c, S)) return rc;
  if (K > 0 && probes)
    cudaMemcpyAsync(L->zp, probes, sizeof(float) * (size_t)K * S.n, cudaMemcpyHostToDevice, s);
  else if (K > 0)
    k_probes<<<lv_blocks(S.n, TPB), TPB, 0, s>>>(S.n, K, seed, L->zp);
  if (int rc = loss_grad_G(c, S, K)) return rc;
  if (int rc = backward(c, S)) return rc;
  if (loss) cudaMemcpyAsync(loss, L->loss, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (grad) cudaMemcpyAsync(grad, L->grad, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, s);
  return lv_cuda_check(c, cudaStreamSynchronize(s), "lv_learn_loss_grad");
}

// Adam on the training systems (round robin), K Rademacher probes per step.
int lv_learn_train(lv_ctx* c, int32_t steps, float lr, int32_t K, uint64_t seed, float* losses) {
  if (c) c->factor_valid = false;
  if (!c || steps < 0 || K < 0 || K > MAXPROBES || !(lr > 0)) return LV_ERR_BAD_ARGUMENT;
  if (int rc = ensure_state(c)) return rc;
  LearnState* L = c->learn;
  if (K > 0 && L->hops == 2)
    return lv_fail(c, LV_ERR_BAD_ARGUMENT, "the Hutchinson objective supports the one-hop pattern only");
  if (L->systems.empty()) return lv_fail(c, LV_ERR_BAD_ARGUMENT, "no training systems (lv_learn_add_system)");
  cudaStream_t s = c->stream;
  std::vector<double> hl(steps > 0 ? steps : 1);
  double* dl = nullptr;
  if (losses && steps > 0 && cudaMalloc(&dl, sizeof(double) * steps) != cudaSuccess) dl = nullptr;
  for (int st = 0; st < steps; ++st) {
    const LearnSystem& S = L->systems[st % L->systems.size()];
    if (int rc = prepare(c, S)) return rc;
    if (int rc = forward(c, S)) return rc;
    if (K > 0) k_probes<<<lv_blocks(S.n, TPB), TPB, 0, s>>>(S.n, K, seed + 7919ull * (unsigned long long)st, L->zp);
    if (int rc = loss_grad_G(c, S, K)) return rc;
    if (int rc = backward(c, S)) return rc;
    L->adam_t += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)L->adam_t), c2 = 1.f - powf(b2, (float)L->adam_t);
    k_adam<<<lv_blocks(NPARAM, TPB), TPB, 0, s>>>(NPARAM, L->params, L->grad, L->m1, L->m2, lr, b1, b2, c1, c2);
    L->wbf_valid = false;
    c->launches += 2;
    if (dl) cudaMemcpyAsync(dl + st, L->loss, sizeof(double), cudaMemcpyDeviceToDevice, s);
  }
  if (dl) {
    cudaMemcpyAsync(hl.data(), dl, sizeof(double) * steps, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    for (int st = 0; st < steps; ++st) losses[st] = (float)hl[st];
    cudaFree(dl);
  }
  L->factor_ready = true;
  return lv_cuda_check(c, cudaStreamSynchronize(s), "lv_learn_train");
}

// Pattern of the learned factor: 1 = the operator's lower triangle, 2 = also
// the lower two-hop neighbours.
int lv_learn_set_pattern(lv_ctx* c, int32_t hops) {
  if (!c || (hops != 1 && hops != 2)) return LV_ERR_BAD_ARGUMENT;
  if (int rc = ensure_state(c)) return rc;
  c->learn->hops = hops;
  c->factor_valid = false;
  if (hops == 2) return ensure_hop2(c);
  return LV_OK;
}

int32_t lv_learn_get_pattern(lv_ctx* c) { return (c && c->learn) ? c->learn->hops : 1; }

// The two-hop part of the current factor: the two-hop pattern as a CSR
// (rowptr2[n+1], col2[nnz2]) and its values g2[nnz2] (lower entries, zero
// elsewhere); with NULL arrays only *nnz2 is returned.
int lv_learn_factor2(lv_ctx* c, int64_t* nnz2, int64_t* rowptr2, int32_t* col2, float* g2) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  if (!c->op_ready) return lv_fail(c, LV_ERR_NOT_MESHED, "the pressure operator has not been assembled");
  if (int rc = ensure_state(c)) return rc;
  LearnState* L = c->learn;
  if (L->hops != 2) return lv_fail(c, LV_ERR_BAD_ARGUMENT, "the factor has the one-hop pattern");
  if (int rc = lv_learn_factor_current(c)) return rc;
  const int n = c->n;
  std::vector<int> rp(n + 1);
  cudaMemcpyAsync(rp.data(), L->rowptr2, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, c->stream);
  cudaStreamSynchronize(c->stream);
  if (nnz2) *nnz2 = rp[n];
  if (rowptr2)
    for (int i = 0; i <= n; ++i) rowptr2[i] = rp[i];
  if (col2) cudaMemcpyAsync(col2, L->col2, sizeof(int) * rp[n], cudaMemcpyDeviceToHost, c->stream);
  if (g2) cudaMemcpyAsync(g2, L->gl2, sizeof(float) * rp[n], cudaMemcpyDeviceToHost, c->stream);
  return lv_cuda_check(c, cudaStreamSynchronize(c->stream), "lv_learn_factor2");
}

// The factor Gt of the current operator: gdiag[n] and glower[nnz] (entries of
// the CSR positions with col < row; others 0), plus the features X[n][16].
int lv_learn_factor(lv_ctx* c, float* gdiag, float* glower, float* features) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  if (!c->op_ready) return lv_fail(c, LV_ERR_NOT_MESHED, "the pressure operator has not been assembled");
  if (int rc = lv_learn_factor_current(c)) return rc;
  LearnState* L = c->learn;
  int nnz = 0;
  cudaMemcpyAsync(&nnz, c->sv.rowptr + c->n, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  cudaStreamSynchronize(c->stream);
  if (gdiag) cudaMemcpyAsync(gdiag, L->gd, sizeof(float) * c->n, cudaMemcpyDeviceToHost, c->stream);
  if (glower) cudaMemcpyAsync(glower, L->gl, sizeof(float) * nnz, cudaMemcpyDeviceToHost, c->stream);
  if (features) cudaMemcpyAsync(features, L->X, sizeof(float) * c->n * FIN, cudaMemcpyDeviceToHost, c->stream);
  return lv_cuda_check(c, cudaStreamSynchronize(c->stream), "lv_learn_factor");
}

}  // extern "C"
