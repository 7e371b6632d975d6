// C ABI of liblvgpu (include/lvgpu.h): context, device memory, transfers and
// the entry points that sequence the kernels of lv_mesh.cu, lv_physics.cu
// and lv_solver.cu on the context's stream.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "lv_internal.cuh"

int lv_fail(lv_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int lv_cuda_check(lv_ctx* c, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return LV_OK;
  return lv_fail(c, LV_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

namespace {

template <class T>
T* dalloc(lv_ctx* c, size_t count, bool* ok) {
  void* p = nullptr;
  if (count == 0) count = 1;
  if (cudaMalloc(&p, sizeof(T) * count) != cudaSuccess) {
    *ok = false;
    return nullptr;
  }
  cudaMemset(p, 0, sizeof(T) * count);
  c->allocs.push_back(p);
  return static_cast<T*>(p);
}

// neighborlist.jl:29-41: the visited prefix of the cell path (every node with
// rr <= rr_max, then the first node beyond, at which the search either stops
// or reports a destroyed mesh); offsets range over the reference's swapped
// bounds i1 in [1-n2, n2-1], i2 in [1-n1, n1-1]; order = stable sort by |key|^2,
// then stable sort by rr.
std::vector<PathNodeDev> build_path(const GridDev& g) {
  struct Node {
    long long i1, i2, keysq;
    double rr;
  };
  const long long R = (long long)ceil(sqrt(g.rr_max) / g.h) + 3;
  const long long lo2 = std::max<long long>(1 - (long long)g.n1, -R), hi2 = std::min<long long>(g.n1 - 1, R);
  const long long lo1 = std::max<long long>(1 - (long long)g.n2, -R), hi1 = std::min<long long>(g.n2 - 1, R);
  std::vector<Node> all;
  for (long long i2 = lo2; i2 <= hi2; ++i2)
    for (long long i1 = lo1; i1 <= hi1; ++i1) {
      long long a = std::max<long long>(0, llabs(i1) - 1), b = std::max<long long>(0, llabs(i2) - 1);
      volatile double hh = g.h * g.h;  // keep (h*h)*k, as the reference's h^2*(...)
      double rr = hh * (double)(a * a + b * b);
      all.push_back({i1, i2, i1 * i1 + i2 * i2, rr});
    }
  std::stable_sort(all.begin(), all.end(), [](const Node& p, const Node& q) { return p.keysq < q.keysq; });
  std::stable_sort(all.begin(), all.end(), [](const Node& p, const Node& q) { return p.rr < q.rr; });
  std::vector<PathNodeDev> out;
  for (const auto& nd : all) {
    out.push_back(PathNodeDev{(int)nd.i1, (int)nd.i2, nd.rr, (float)nd.rr, nd.rr > g.rr_max ? 1 : 0});
    if (nd.rr > g.rr_max) break;
  }
  return out;
}

}  // namespace

// Function attributes (dynamic shared memory beyond 48 KB, carveouts) belong
// to a device: they are set once per device, by the first context created on
// it, whichever host thread that is.
int lv_device_setup(int dev) {
  static std::once_flag once[LV_MAX_DEVICES];
  static int rc[LV_MAX_DEVICES];
  if (dev < 0 || dev >= LV_MAX_DEVICES) return LV_ERR_BAD_ARGUMENT;
  std::call_once(once[dev], [dev]() {
    int r = lv_mesh_device_setup();
    if (r == LV_OK) r = lv_fcg_device_setup();
    if (r == LV_OK) r = lv_learn_device_setup();
    rc[dev] = r;
  });
  return rc[dev];
}

namespace {

int nimages(const GridDev& g) { return 1 + (g.xper ? 2 : 0) + (g.yper ? 2 : 0) + ((g.xper && g.yper) ? 4 : 0); }

int decode_status(int flags) {
  // root causes first: a cell list that overflowed leaves candidates out of
  // the clip, which can also destroy the mesh or overflow a polygon
  if (flags & LV_FLAG_NAN_VELOCITY) return LV_ERR_NAN_VELOCITY;
  if (flags & LV_FLAG_NONFINITE) return LV_ERR_NONFINITE_POSITION;
  if (flags & LV_FLAG_CELL_OVERFLOW) return LV_ERR_CELL_OVERFLOW;
  if (flags & LV_FLAG_MESH_DESTROYED) return LV_ERR_MESH_DESTROYED;
  if (flags & LV_FLAG_EDGE_OVERFLOW) return LV_ERR_EDGE_OVERFLOW;
  if (flags & LV_FLAG_BARRIER_TIMEOUT) return LV_ERR_BARRIER_TIMEOUT;
  if (flags & LV_FLAG_BAD_INPUT) return LV_ERR_BAD_ARGUMENT;
  return LV_OK;
}

const char* status_message(int code) {
  switch (code) {
    case LV_ERR_NAN_VELOCITY: return "Velocity field invalidated.";
    case LV_ERR_MESH_DESTROYED: return "The Voronoi Mesh has been destroyed.";
    case LV_ERR_EDGE_OVERFLOW: return "a Voronoi polygon exceeded LV_MAX_EDGES edges";
    case LV_ERR_CELL_OVERFLOW: return "cell list capacity exceeded";
    case LV_ERR_NONFINITE_POSITION: return "non-finite particle position";
    case LV_ERR_BARRIER_TIMEOUT: return "grid barrier timed out in a persistent kernel";
    case LV_ERR_BAD_ARGUMENT: return "heat_from_bdary!: every boundary polygon needs cV > 0";
    default: return "";
  }
}

// Reads and clears the device status word (synchronises the stream).
int sync_status(lv_ctx* c) {
  cudaError_t e = cudaMemcpyAsync(c->status_host, c->status, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return lv_cuda_check(c, e, "stream synchronize");
  int flags = *c->status_host;
  if (flags & LV_FLAG_BARRIER_TIMEOUT) {
    // a solver launch stopped part-way: its synchronisation words start
    // afresh, and the sweeps' history (partly written) is dropped
    c->fcg_reset = c->big_reset = c->mr_reset = true;
    c->sg_valid = 0;
  }
  if (flags) {
    cudaMemsetAsync(c->status, 0, sizeof(int), c->stream);
    int code = decode_status(flags);
    return lv_fail(c, code, status_message(code));
  }
  return LV_OK;
}

struct Timer {
  lv_ctx* c;
  int slot;
  Timer(lv_ctx* cc, int s) : c(cc), slot(s) {
    if (c->timing) cudaEventRecord(c->ev0, c->stream);
  }
  ~Timer() {
    if (c->timing) {
      cudaEventRecord(c->ev1, c->stream);
      cudaEventSynchronize(c->ev1);
      float ms = 0;
      cudaEventElapsedTime(&ms, c->ev0, c->ev1);
      c->t_ms[slot] += ms;
    }
  }
};

__global__ void k_split_phase(const double* __restrict__ src, int* dst, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (int)src[i];
}

// Queue one field transfer on the context's stream (no synchronisation).
int queue_set_field(lv_ctx* c, int32_t f, const double* h);
int queue_get_field(lv_ctx* c, int32_t f, double* h, std::vector<int>* phase_tmp);

}  // namespace

KernelTimer::KernelTimer(lv_ctx* cc, int f) : c(cc), fam(f) {
  if (!c->ktiming) return;
  auto& k = c->kev[fam];
  if (k.used + 2 > k.ev.size()) {
    for (int t = 0; t < 64; ++t) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      k.ev.push_back(e);
    }
  }
  cudaEventRecord(k.ev[k.used], c->stream);
}

KernelTimer::~KernelTimer() {
  if (!c->ktiming) return;
  auto& k = c->kev[fam];
  cudaEventRecord(k.ev[k.used + 1], c->stream);
  k.used += 2;
  k.launches += 1;
}

extern "C" {

lv_ctx* lv_create(const lv_params* prm) {
  if (!prm || prm->capacity <= 0 || !(prm->dr > 0)) return nullptr;
  if (!(prm->xmax[0] > prm->xmin[0]) || !(prm->xmax[1] > prm->xmin[1])) return nullptr;
  lv_ctx* c = new lv_ctx();
  c->prm = *prm;
  c->dev = prm->device;
  if (cudaSetDevice(c->dev) != cudaSuccess) {
    delete c;
    return nullptr;
  }
  GridDev& g = c->g;
  const double dr = prm->dr;
  const double h = prm->h > 0 ? prm->h : 2.0 * dr;
  const double r_max = prm->r_max > 0 ? prm->r_max : 10.0 * dr;
  g.dr = dr;
  g.h = h;
  g.rh = 1.0 / h;
  g.xper = prm->xperiodic ? 1 : 0;
  g.yper = prm->yperiodic ? 1 : 0;
  g.bminx = prm->xmin[0];
  g.bminy = prm->xmin[1];
  g.bmaxx = prm->xmax[0];
  g.bmaxy = prm->xmax[1];
  // voronoigrid.jl:29-33: cropping rectangle enlarged by r_max in periodic directions
  const double rx = g.xper ? r_max : 0.0, ry = g.yper ? r_max : 0.0;
  g.cminx = g.bminx - rx;
  g.cminy = g.bminy - ry;
  g.cmaxx = g.bmaxx + rx;
  g.cmaxy = g.bmaxy + ry;
  g.xperiod = g.bmaxx - g.bminx;
  g.yperiod = g.bmaxy - g.bminy;
  g.rr_max = r_max * r_max;
  // neighborlist.jl:18-27
  g.ox = g.cminx - h;
  g.oy = g.cminy - h;
  g.n1 = (int)floor((g.cmaxx - g.cminx) / h) + 3;
  g.n2 = (int)floor((g.cmaxy - g.cminy) / h) + 3;
  // dx >= dx_hi implies floor(dx / h) >= n1 whatever the rounding of the quotient
  g.dx_hi = (double)g.n1 * h * (1.0 + 1e-12);
  g.dy_hi = (double)g.n2 * h * (1.0 + 1e-12);
  const double bigm = std::max(std::max(fabs(g.cminx), fabs(g.cmaxx)), std::max(fabs(g.cminy), fabs(g.cmaxy)));
  g.bigm = (float)(bigm * (1.0 + 1e-6));
  c->path_host = build_path(g);
  g.npath = (int)c->path_host.size();
  // The clipping's float candidate offset from the seed is
  //   ((cpos - float(x - O_seedcell)) + float(di) * float(h)),
  // each offset in [0, h] rounded once to FP64 and once to float.  Its error
  // per component is at most 2^-24 h (4 + 3 |di|) (two offsets, their
  // difference, the product and the sum, each a float rounding) plus the FP64
  // rounding of the cell corners and of the reference's arrow (a few ulps of
  // the largest coordinate); |di| <= dmax over the nodes the search visits.
  int dmax = 0;
  for (const PathNodeDev& nd : c->path_host)
    if (!nd.beyond) dmax = std::max(dmax, std::max(abs(nd.di1), abs(nd.di2)));
  g.h32 = (float)h;
  // four cell sizes of margin: the grid ends 2h past the cropping box, and
  // the float rounding of a position is far below h
  g.ixlo = (float)(g.bminx + r_max + 4.0 * h);
  g.ixhi = (float)(g.bmaxx - r_max - 4.0 * h);
  g.iylo = (float)(g.bminy + r_max + 4.0 * h);
  g.iyhi = (float)(g.bmaxy - r_max - 4.0 * h);
  {
    const double hxp = 0.5 * g.xperiod, hyp = 0.5 * g.yperiod;
    memcpy(&g.hxbits, &hxp, sizeof(double));
    memcpy(&g.hybits, &hyp, sizeof(double));
  }
  g.delta32 = (float)((ldexp(1.0, -24) * h * (6.0 + 4.0 * dmax) +
                       2e-15 * (bigm + std::max(g.xperiod, g.yperiod) + 2.0 * h)) * (1.0 + 1e-6));

  cudaDeviceProp p;
  cudaGetDeviceProperties(&p, c->dev);
  c->num_sms = p.multiProcessorCount;
  if (!p.cooperativeLaunch) {
    delete c;
    return nullptr;
  }
  cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  cudaEventCreate(&c->ev0);
  cudaEventCreate(&c->ev1);
  const char* tenv = getenv("LVGPU_TIMING");
  c->timing = tenv && tenv[0] == '1';
  // test knobs, read once here: the first clipping pass's edge slots, the
  // sweep guess, a lowered cell-list capacity
  if (const char* env = getenv("LVGPU_CLIP_SLOTS")) c->clip_slots = atoi(env);
  const char* sgenv = getenv("LVGPU_SWEEP_GUESS");
  c->sweep_guess = !(sgenv && sgenv[0] == '0');
  long long cell_items = 0;
  if (const char* env = getenv("LVGPU_CELL_ITEMS")) cell_items = atoll(env);
  // function attributes are per device: set them once for this one
  if (c->dev < 0 || c->dev >= LV_MAX_DEVICES || lv_device_setup(c->dev) != LV_OK) {
    cudaStreamDestroy(c->stream);
    cudaEventDestroy(c->ev0);
    cudaEventDestroy(c->ev1);
    delete c;
    return nullptr;
  }

  const int cap = (prm->capacity + 31) / 32 * 32;
  c->cap = cap;
  bool ok = true;
  StateDev& s = c->s;
  s.x = dalloc<double2>(c, cap, &ok);
  s.v = dalloc<double2>(c, cap, &ok);
  s.dv = dalloc<double2>(c, cap, &ok);
  s.mom = dalloc<double2>(c, cap, &ok);
  s.Da = dalloc<double2>(c, cap, &ok);
  s.Db = dalloc<double2>(c, cap, &ok);
  s.GP = dalloc<double2>(c, cap, &ok);
  s.e = dalloc<double>(c, cap, &ok);
  s.P = dalloc<double>(c, cap, &ok);
  s.rho = dalloc<double>(c, cap, &ok);
  s.c2 = dalloc<double>(c, cap, &ok);
  s.mass = dalloc<double>(c, cap, &ok);
  s.energy = dalloc<double>(c, cap, &ok);
  s.quality = dalloc<double>(c, cap, &ok);
  s.mu = dalloc<double>(c, cap, &ok);
  s.T = dalloc<double>(c, cap, &ok);
  s.kc = dalloc<double>(c, cap, &ok);
  s.cV = dalloc<double>(c, cap, &ok);
  s.phase = dalloc<int>(c, cap, &ok);

  MeshDev& m = c->m;
  m.cap = cap;
  const size_t ell = (size_t)LV_MAX_EDGES * cap;
  m.nedges = dalloc<int>(c, cap, &ok);
  m.nfaces = dalloc<int>(c, cap + 1, &ok);
  m.ev1 = dalloc<double2>(c, ell, &ok);
  m.ev2 = dalloc<double2>(c, ell, &ok);
  m.elab = dalloc<int>(c, ell, &ok);
  m.fnbr = dalloc<int>(c, ell, &ok);
  m.flrr = dalloc<double>(c, ell, &ok);
  m.flen = dalloc<double>(c, ell, &ok);
  m.fm = dalloc<double2>(c, ell, &ok);
  m.fy = dalloc<double2>(c, ell, &ok);
  m.area = dalloc<double>(c, cap, &ok);
  m.rperm = dalloc<int>(c, cap, &ok);
  m.nclip = dalloc<unsigned char>(c, cap, &ok);
  m.cperm = dalloc<int>(c, cap, &ok);
  m.centroid = dalloc<double2>(c, cap, &ok);

  CellsDev& cl = c->c;
  cl.ncells = g.n1 * g.n2;
  cl.cstart = dalloc<int>(c, (size_t)cl.ncells + 1, &ok);
  cl.ccount = dalloc<int>(c, cl.ncells, &ok);
  // every copy of every seed has a cell-list slot, so the list cannot
  // overflow; LVGPU_CELL_ITEMS (tests) lowers its capacity to inject that
  // error (the per-copy keys keep one entry per copy)
  const int copies = cap * nimages(g);
  cl.item_cap = copies;
  if (cell_items > 0 && cell_items < cl.item_cap) cl.item_cap = (int)cell_items;
  cl.citem = dalloc<int>(c, cl.item_cap, &ok);
  cl.bkey = dalloc<int2>(c, copies, &ok);
  cl.cpos = dalloc<float2>(c, cl.item_cap, &ok);

  SolverDev& sv = c->sv;
  sv.nnz_cap = (int64_t)ell;
  sv.rowptr = dalloc<int>(c, cap + 1, &ok);
  sv.col = dalloc<int>(c, ell, &ok);
  sv.w = dalloc<double>(c, ell, &ok);
  sv.w32 = dalloc<float>(c, ell, &ok);
  sv.diag = dalloc<double>(c, cap, &ok);
  sv.adiag = dalloc<double>(c, cap, &ok);
  sv.dinv = dalloc<double>(c, cap, &ok);
  sv.b = dalloc<double>(c, cap, &ok);
  sv.xs = dalloc<double>(c, cap, &ok);
  sv.pprev = dalloc<double>(c, cap, &ok);
  sv.bprev = dalloc<double>(c, cap, &ok);
  sv.sgd32 = dalloc<float>(c, cap, &ok);
  sv.sgpart = dalloc<double>(c, LV_SG_SUMS * ((size_t)cap / 256 + 2), &ok);
  sv.sgomega = dalloc<double>(c, 2, &ok);
  sv.dinc = nullptr;
  sv.dinc_slots = 0;
  sv.r = dalloc<double>(c, 2 * (size_t)cap, &ok);
  sv.z = dalloc<double>(c, cap, &ok);
  sv.p = dalloc<double>(c, 2 * (size_t)cap, &ok);
  sv.q = dalloc<double>(c, cap, &ok);
  const size_t tmp_n = std::max<size_t>(3 * (size_t)cap, (size_t)cl.ncells / 512 + 64);
  sv.tmp = dalloc<double>(c, tmp_n, &ok);
  sv.dinv32 = dalloc<float>(c, cap, &ok);
  sv.r32 = dalloc<float>(c, cap, &ok);
  sv.rtag = dalloc<unsigned long long>(c, cap, &ok);
  sv.z32 = dalloc<float>(c, cap, &ok);
  sv.p32 = dalloc<float>(c, cap, &ok);
  sv.q32 = dalloc<float>(c, cap, &ok);
  sv.d32 = dalloc<float>(c, cap, &ok);
  sv.e32 = dalloc<float>(c, cap, &ok);
  sv.f32a = dalloc<float>(c, cap, &ok);
  sv.f32b = dalloc<float>(c, cap, &ok);
  sv.part = dalloc<double>(c, 8 * 4096, &ok);
  sv.fslots = dalloc<unsigned long long>(c, LV_FCG_SLOT_WORDS, &ok);
  sv.rhs_tf = dalloc<double>(c, ell, &ok);
  sv.rhs_dmz = dalloc<double2>(c, ell, &ok);
  sv.rhs_te = dalloc<double>(c, ell, &ok);
  sv.rhs_dm = dalloc<double2>(c, ell, &ok);
  sv.rhs_den = dalloc<double>(c, cap, &ok);
  sv.rhs_rden = dalloc<double>(c, cap, &ok);
  sv.rhs_rm = dalloc<double>(c, cap, &ok);
  sv.counters = dalloc<long long>(c, 4, &ok);
  sv.bar = dalloc<unsigned>(c, 4, &ok);
  sv.iters = dalloc<int>(c, LV_IT_SIZE, &ok);
  sv.dstats = dalloc<double>(c, 3 * 64, &ok);
  c->status = dalloc<int>(c, 1, &ok);
  c->path = dalloc<PathNodeDev>(c, c->path_host.size(), &ok);
  if (cudaMallocHost(&c->status_host, sizeof(int)) != cudaSuccess) ok = false;
  if (!ok) {
    lv_destroy(c);
    return nullptr;
  }
  cudaMemcpy(c->path, c->path_host.data(), sizeof(PathNodeDev) * c->path_host.size(), cudaMemcpyHostToDevice);
  cudaDeviceSynchronize();
  return c;
}

int lv_destroy(lv_ctx* c) {
  if (!c) return LV_OK;
  cudaSetDevice(c->dev);
  if (c->stream) cudaStreamSynchronize(c->stream);
  lv_learn_free(c);
  lv_fcg_free(c);
  cudaFree(c->sv.dinc);
  for (void* p : c->allocs) cudaFree(p);
  if (c->status_host) cudaFreeHost(c->status_host);
  if (c->ev0) cudaEventDestroy(c->ev0);
  for (auto& k : c->kev)
    for (cudaEvent_t e : k.ev) cudaEventDestroy(e);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return LV_OK;
}

const char* lv_last_error(const lv_ctx* c) { return c ? c->err.c_str() : "null context"; }

int lv_status(lv_ctx* c) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  return sync_status(c);
}

int lv_synchronize(lv_ctx* c) { return lv_status(c); }

int lv_set_positions(lv_ctx* c, int32_t n, const double* x) {
  if (!c || n < 0 || (n > 0 && !x)) return LV_ERR_BAD_ARGUMENT;
  if (n > c->prm.capacity) return lv_fail(c, LV_ERR_BAD_ARGUMENT, "more particles than the context capacity");
  c->n = n;
  cudaStream_t s = c->stream;
  StateDev& st = c->s;
  const size_t cap = c->cap;
  for (double2* p : {st.x, st.v, st.dv, st.mom, st.Da, st.Db, st.GP}) cudaMemsetAsync(p, 0, 16 * cap, s);
  for (double* p : {st.e, st.P, st.rho, st.c2, st.mass, st.energy, st.quality, st.mu, st.T, st.kc, st.cV})
    cudaMemsetAsync(p, 0, 8 * cap, s);
  cudaMemsetAsync(st.phase, 0, 4 * cap, s);
  cudaError_t e = cudaMemcpyAsync(st.x, x, 16 * (size_t)n, cudaMemcpyHostToDevice, s);
  c->meshed = false;
  c->op_ready = false;
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return lv_cuda_check(c, e, "lv_set_positions");
}

int32_t lv_num_particles(const lv_ctx* c) { return c ? c->n : 0; }

static double* dptr1(lv_ctx* c, int f) {
  StateDev& s = c->s;
  switch (f) {
    case LV_FIELD_E: return s.e;
    case LV_FIELD_P: return s.P;
    case LV_FIELD_RHO: return s.rho;
    case LV_FIELD_C2: return s.c2;
    case LV_FIELD_MASS: return s.mass;
    case LV_FIELD_ENERGY: return s.energy;
    case LV_FIELD_QUALITY: return s.quality;
    case LV_FIELD_MU: return s.mu;
    case LV_FIELD_T: return s.T;
    case LV_FIELD_K: return s.kc;
    case LV_FIELD_CV: return s.cV;
    case LV_FIELD_AREA: return c->m.area;
    default: return nullptr;
  }
}
static double2* dptr2(lv_ctx* c, int f) {
  StateDev& s = c->s;
  switch (f) {
    case LV_FIELD_X: return s.x;
    case LV_FIELD_V: return s.v;
    case LV_FIELD_DV: return s.dv;
    case LV_FIELD_MOMENTUM: return s.mom;
    case LV_FIELD_CENTROID: return c->m.centroid;
    default: return nullptr;
  }
}

int lv_set_fields(lv_ctx* c, int32_t count, const int32_t* fields, const double* const* data) {
  if (!c || count < 0 || (count > 0 && (!fields || !data))) return LV_ERR_BAD_ARGUMENT;
  for (int k = 0; k < count; ++k) {
    if (!data[k]) return LV_ERR_BAD_ARGUMENT;
    if (int rc = queue_set_field(c, fields[k], data[k])) return rc;
  }
  return lv_cuda_check(c, cudaStreamSynchronize(c->stream), "lv_set_fields");
}

int lv_get_fields(lv_ctx* c, int32_t count, const int32_t* fields, double* const* data) {
  if (!c || count < 0 || (count > 0 && (!fields || !data))) return LV_ERR_BAD_ARGUMENT;
  std::vector<std::vector<int>> ph(count);
  for (int k = 0; k < count; ++k) {
    if (!data[k]) return LV_ERR_BAD_ARGUMENT;
    if (int rc = queue_get_field(c, fields[k], data[k], &ph[k])) return rc;
  }
  cudaError_t e = cudaStreamSynchronize(c->stream);
  for (int k = 0; k < count; ++k)
    for (size_t i = 0; i < ph[k].size(); ++i) data[k][i] = ph[k][i];
  return lv_cuda_check(c, e, "lv_get_fields");
}

int lv_set_field(lv_ctx* c, int32_t f, const double* h) {
  if (!c || !h) return LV_ERR_BAD_ARGUMENT;
  if (int rc = queue_set_field(c, f, h)) return rc;
  return lv_cuda_check(c, cudaStreamSynchronize(c->stream), "lv_set_field");
}

int lv_get_field(lv_ctx* c, int32_t f, double* h) {
  if (!c || !h) return LV_ERR_BAD_ARGUMENT;
  std::vector<int> ph;
  if (int rc = queue_get_field(c, f, h, &ph)) return rc;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  for (size_t i = 0; i < ph.size(); ++i) h[i] = ph[i];
  return lv_cuda_check(c, e, "lv_get_field");
}

}  // extern "C"

namespace {

int queue_set_field(lv_ctx* c, int32_t f, const double* h) {
  const size_t n = c->n;
  cudaStream_t s = c->stream;
  cudaError_t e = cudaSuccess;
  if (f == LV_FIELD_AREA || f == LV_FIELD_CENTROID)
    return lv_fail(c, LV_ERR_BAD_ARGUMENT, "geometry fields are read-only");
  if (double* d = dptr1(c, f)) {
    e = cudaMemcpyAsync(d, h, 8 * n, cudaMemcpyHostToDevice, s);
  } else if (double2* d2 = dptr2(c, f)) {
    e = cudaMemcpyAsync(d2, h, 16 * n, cudaMemcpyHostToDevice, s);
    if (f == LV_FIELD_X) {
      c->meshed = false;
      c->op_ready = false;
    }
  } else if (f == LV_FIELD_D) {
    e = cudaMemcpy2DAsync(c->s.Da, 16, h, 32, 16, n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpy2DAsync(c->s.Db, 16, h + 2, 32, 16, n, cudaMemcpyHostToDevice, s);
  } else if (f == LV_FIELD_PHASE) {
    double* tmp = c->sv.tmp;
    e = cudaMemcpyAsync(tmp, h, 8 * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && n > 0) {
      k_split_phase<<<lv_blocks((int)n, 256), 256, 0, s>>>(tmp, c->s.phase, (int)n);
      c->launches++;
      e = cudaGetLastError();
    }
  } else {
    return lv_fail(c, LV_ERR_BAD_ARGUMENT, "unknown field");
  }
  return lv_cuda_check(c, e, "lv_set_field");
}

// phase (int32 on the device) lands in *phase_tmp, converted by the caller
// after the synchronisation
int queue_get_field(lv_ctx* c, int32_t f, double* h, std::vector<int>* phase_tmp) {
  const size_t n = c->n;
  cudaStream_t s = c->stream;
  cudaError_t e = cudaSuccess;
  if (double* d = dptr1(c, f)) {
    e = cudaMemcpyAsync(h, d, 8 * n, cudaMemcpyDeviceToHost, s);
  } else if (double2* d2 = dptr2(c, f)) {
    e = cudaMemcpyAsync(h, d2, 16 * n, cudaMemcpyDeviceToHost, s);
  } else if (f == LV_FIELD_D) {
    e = cudaMemcpy2DAsync(h, 32, c->s.Da, 16, 16, n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpy2DAsync(h + 2, 32, c->s.Db, 16, 16, n, cudaMemcpyDeviceToHost, s);
  } else if (f == LV_FIELD_PHASE) {
    phase_tmp->resize(n);
    e = cudaMemcpyAsync(phase_tmp->data(), c->s.phase, 4 * n, cudaMemcpyDeviceToHost, s);
  } else {
    return lv_fail(c, LV_ERR_BAD_ARGUMENT, "unknown field");
  }
  return lv_cuda_check(c, e, "lv_get_field");
}

}  // namespace

extern "C" {

void* lv_field_device_ptr(lv_ctx* c, int32_t f) {
  if (!c) return nullptr;
  if (double* d = dptr1(c, f)) return d;
  if (double2* d2 = dptr2(c, f)) return d2;
  if (f == LV_FIELD_PHASE) return c->s.phase;
  return nullptr;
}

int lv_remesh_async(lv_ctx* c) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  Timer t(c, 0);
  return lv_mesh_remesh(c);
}

int lv_remesh(lv_ctx* c) {
  int rc = lv_remesh_async(c);
  if (rc) return rc;
  return sync_status(c);
}

int lv_get_geometry(lv_ctx* c, int32_t* nedges, double* verts, int32_t* labels) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  if (!c->meshed) return lv_fail(c, LV_ERR_NOT_MESHED, "the grid has not been meshed");
  const int n = c->n, cap = c->cap;
  std::vector<int> ne(n);
  cudaStream_t s = c->stream;
  cudaMemcpyAsync(ne.data(), c->m.nedges, 4 * n, cudaMemcpyDeviceToHost, s);
  std::vector<double2> v1, v2;
  std::vector<int> lab;
  if (verts) {
    v1.resize((size_t)LV_MAX_EDGES * cap);
    v2.resize((size_t)LV_MAX_EDGES * cap);
    cudaMemcpyAsync(v1.data(), c->m.ev1, 16 * v1.size(), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(v2.data(), c->m.ev2, 16 * v2.size(), cudaMemcpyDeviceToHost, s);
  }
  if (labels) {
    lab.resize((size_t)LV_MAX_EDGES * cap);
    cudaMemcpyAsync(lab.data(), c->m.elab, 4 * lab.size(), cudaMemcpyDeviceToHost, s);
  }
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return lv_cuda_check(c, e, "lv_get_geometry");
  for (int i = 0; i < n; ++i) {
    if (nedges) nedges[i] = ne[i];
    for (int k = 0; k < ne[i] && k < LV_MAX_EDGES; ++k) {
      const size_t src = (size_t)k * cap + i, dst = (size_t)i * LV_MAX_EDGES + k;
      if (verts) {
        verts[4 * dst] = v1[src].x;
        verts[4 * dst + 1] = v1[src].y;
        verts[4 * dst + 2] = v2[src].x;
        verts[4 * dst + 3] = v2[src].y;
      }
      if (labels) labels[dst] = lab[src];
    }
  }
  return LV_OK;
}

int lv_get_faces(lv_ctx* c, int64_t* nfaces, int64_t* rowptr, int32_t* nbr, double* lrr, double* mid, double* y,
                 double* len) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  if (!c->meshed) return lv_fail(c, LV_ERR_NOT_MESHED, "the grid has not been meshed");
  const int n = c->n, cap = c->cap;
  cudaStream_t s = c->stream;
  std::vector<int> nf(n);
  cudaMemcpyAsync(nf.data(), c->m.nfaces, 4 * n, cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return lv_cuda_check(c, e, "lv_get_faces");
  int64_t tot = 0;
  for (int i = 0; i < n; ++i) tot += nf[i];
  if (nfaces) *nfaces = tot;
  if (!rowptr && !nbr) return LV_OK;
  if (int rc = lv_mesh_face_len(c)) return rc;
  const size_t ell = (size_t)LV_MAX_EDGES * cap;
  std::vector<int> fn(ell);
  std::vector<double> fl(ell), fle(ell);
  std::vector<double2> fm(ell), fy(ell);
  cudaMemcpyAsync(fn.data(), c->m.fnbr, 4 * ell, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(fl.data(), c->m.flrr, 8 * ell, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(fle.data(), c->m.flen, 8 * ell, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(fm.data(), c->m.fm, 16 * ell, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(fy.data(), c->m.fy, 16 * ell, cudaMemcpyDeviceToHost, s);
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return lv_cuda_check(c, e, "lv_get_faces");
  int64_t k = 0;
  for (int i = 0; i < n; ++i) {
    if (rowptr) rowptr[i] = k;
    for (int t = 0; t < nf[i]; ++t, ++k) {
      const size_t src = (size_t)t * cap + i;
      if (nbr) nbr[k] = fn[src];
      if (lrr) lrr[k] = fl[src];
      if (len) len[k] = fle[src];
      if (mid) {
        mid[2 * k] = fm[src].x;
        mid[2 * k + 1] = fm[src].y;
      }
      if (y) {
        y[2 * k] = fy[src].x;
        y[2 * k + 1] = fy[src].y;
      }
    }
  }
  if (rowptr) rowptr[n] = k;
  return LV_OK;
}

int lv_get_cell_list(lv_ctx* c, int64_t* ncells, int64_t* nitems, int32_t* starts, int32_t* items) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  const int nc = c->c.ncells;
  if (ncells) *ncells = nc;
  int tot = 0;
  cudaMemcpyAsync(&tot, c->c.cstart + nc, 4, cudaMemcpyDeviceToHost, c->stream);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return lv_cuda_check(c, e, "lv_get_cell_list");
  if (nitems) *nitems = tot;
  if (starts) cudaMemcpyAsync(starts, c->c.cstart, 4 * ((size_t)nc + 1), cudaMemcpyDeviceToHost, c->stream);
  if (items) cudaMemcpyAsync(items, c->c.citem, 4 * (size_t)std::min(tot, c->c.item_cap), cudaMemcpyDeviceToHost, c->stream);
  e = cudaStreamSynchronize(c->stream);
  return lv_cuda_check(c, e, "lv_get_cell_list");
}

// ------------------------------------------------------------ physics

int lv_move(lv_ctx* c, double dt) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  Timer t(c, 0);
  return lv_phys_move(c, dt);
}
int lv_ideal_eos(lv_ctx* c, double gamma, double Pmin) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  Timer t(c, 1);
  return lv_phys_eos(c, 0, gamma, Pmin);
}
int lv_stiffened_eos(lv_ctx* c, double gamma, double P0) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  Timer t(c, 1);
  return lv_phys_eos(c, 1, gamma, P0);
}
int lv_find_rho(lv_ctx* c) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  Timer t(c, 1);
  return lv_phys_eos(c, 2, 0.0, 0.0);
}
int lv_gravity_step(lv_ctx* c, double gx, double gy, double dt) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  Timer t(c, 1);
  return lv_phys_gravity(c, gx, gy, dt);
}
int lv_pressure_step(lv_ctx* c, double dt) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  Timer t(c, 1);
  return lv_phys_pressure_step(c, dt);
}
int lv_find_D(lv_ctx* c) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  Timer t(c, 1);
  return lv_phys_find_D(c);
}
int lv_viscous_step(lv_ctx* c, double dt, int32_t av) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  Timer t(c, 1);
  return lv_phys_viscous(c, dt, av);
}
int lv_bdary_friction(lv_ctx* c, const double* vwall, double dt) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  Timer t(c, 1);
  return lv_phys_friction(c, vwall, dt);
}
int lv_ideal_temperature(lv_ctx* c) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  Timer t(c, 1);
  return lv_phys_ideal_temperature(c);
}
int lv_fourier_step(lv_ctx* c, double dt) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  Timer t(c, 1);
  return lv_phys_fourier(c, dt);
}
int lv_heat_from_bdary_edges(lv_ctx* c, int64_t nb, const double* T_bc, double gamma, double dt) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  (void)gamma;  // the reference's signature carries it; its body uses cV
  Timer t(c, 1);
  return lv_phys_heat_bdary(c, nb, T_bc, dt);
}
int lv_viscous_solve(lv_ctx* c, double dt, lv_solve_stats* stats) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  Timer t(c, 1);
  if (int rc = lv_phys_viscous_implicit(c, dt)) return rc;
  if (!stats) return LV_OK;
  int it = 0, solved = 0;
  double d[3] = {0, 0, 0};
  cudaMemcpyAsync(&it, c->sv.iters + LV_IT_ITERS + LV_VISC_SLOT, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  cudaMemcpyAsync(&solved, c->sv.iters + LV_IT_OUTER + LV_VISC_SLOT, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  cudaMemcpyAsync(d, c->sv.dstats + 3 * LV_VISC_SLOT, sizeof(d), cudaMemcpyDeviceToHost, c->stream);
  if (int rc = sync_status(c)) return rc;
  stats->iterations = it;
  stats->converged = solved;
  stats->outer = 0;
  stats->method = LV_METHOD_MINRES;
  stats->rel_residual = d[1] > 0 ? sqrt(d[0] / d[1]) : sqrt(d[0]);
  return LV_OK;
}
int lv_find_dv(lv_ctx* c, double dt, double alpha) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  Timer t(c, 1);
  return lv_phys_find_dv(c, dt, alpha);
}
int lv_relaxation_step(lv_ctx* c, double dt, int32_t rusanov) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  Timer t(c, 0);
  return lv_phys_relax(c, dt, rusanov);
}

// ------------------------------------------------------------ pressure

int lv_set_solver(lv_ctx* c, int32_t method, double tol, int32_t itmax) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  if (method < LV_METHOD_JACOBI_PCG || method > LV_METHOD_MINRES || !(tol > 0) || itmax <= 0)
    return lv_fail(c, LV_ERR_BAD_ARGUMENT, "lv_set_solver: bad method, tol or itmax");
  c->method = method;
  c->tol = tol;
  c->itmax = itmax;
  return LV_OK;
}

int lv_pressure_operator(lv_ctx* c, double dt) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  Timer t(c, 2);
  return lv_solver_assemble(c, dt);
}

int lv_pressure_rhs(lv_ctx* c, double dt, int32_t gp_step, const double* vbc) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  Timer t(c, 2);
  return lv_phys_rhs(c, dt, gp_step, vbc, 1);
}

static int find_pressure(lv_ctx* c, double dt, int32_t niter, const double* vbc, lv_solve_stats* stats);

int lv_find_pressure(lv_ctx* c, double dt, int32_t niter, const double* vbc, lv_solve_stats* stats) {
  if (!c || niter < 0 || niter > 31) return lv_fail(c, LV_ERR_BAD_ARGUMENT, "niter must be in [0, 31]");
  c->rhs_bvel = nullptr;
  return find_pressure(c, dt, niter, vbc, stats);
}

int lv_find_pressure_edges(lv_ctx* c, double dt, int32_t niter, int64_t nb, const double* vb, lv_solve_stats* stats) {
  if (!c || niter < 0 || niter > 31) return lv_fail(c, LV_ERR_BAD_ARGUMENT, "niter must be in [0, 31]");
  if (int rc = lv_bnd_upload(c, nb, vb, nullptr)) return rc;
  c->rhs_bvel = c->bnd_vel;  // read by the first sweep's right-hand side preparation
  const int rc = find_pressure(c, dt, niter, nullptr, stats);
  c->rhs_bvel = nullptr;
  return rc;
}

int lv_get_boundary_edges(lv_ctx* c, int64_t* nb, double* mid, int32_t* label) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  if (int rc = lv_bnd_prepare(c)) return rc;
  if (nb) *nb = c->bnd_count;
  if (!mid && !label) return LV_OK;
  return lv_bnd_list(c, mid, label);
}

int lv_bdary_friction_edges(lv_ctx* c, int64_t nb, const double* vb, const uint8_t* active, double dt) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  Timer t(c, 1);
  if (int rc = lv_bnd_upload(c, nb, vb, active)) return rc;
  return lv_phys_friction(c, nullptr, dt, c->bnd_vel, active ? c->bnd_act : nullptr);
}

static int find_pressure(lv_ctx* c, double dt, int32_t niter, const double* vbc, lv_solve_stats* stats) {
  Timer t(c, 2);
  c->sg_pending = false;  // a start queued by a call that failed is void
  int rc = lv_solver_assemble(c, dt);
  if (rc) return rc;
  SolverDev& sv = c->sv;
  // MINRES is the reference's solve, warm-started from P as the reference
  // does (pressure.jl:219); the Galerkin start serves the CG methods
  const bool guess = c->sweep_guess && c->method != LV_METHOD_MINRES;
  if (guess && niter > sv.dinc_slots) {
    // one FP32 vector per sweep for the sweeps' changes (kept for the next call)
    cudaFree(sv.dinc);
    sv.dinc = nullptr;
    sv.dinc_slots = 0;
    c->sg_valid = 0;
    if (cudaMalloc(&sv.dinc, sizeof(float) * (size_t)niter * c->cap) != cudaSuccess)
      return lv_fail(c, LV_ERR_CUDA, "allocation of the sweep-guess history failed");
    sv.dinc_slots = niter;
  }
  if (c->sg_n != c->n || !guess) c->sg_valid = 0;
  const size_t cap = (size_t)c->cap;
  for (int it = 1; it <= niter; ++it) {
    // the previous call's change of this sweep, while it is still there
    const float* D = (guess && it <= c->sg_valid) ? sv.dinc + (size_t)(it - 1) * cap : nullptr;
    rc = lv_phys_rhs(c, dt, it > 1, vbc, it == 1, guess ? 1 : 0, D);
    if (rc) return rc;
    if (guess) {
      KernelTimer kt(c, LV_KF_RHS);  // prepares the sweep's system, like the right-hand side
      // this call's change of the previous sweep replaces the old one
      float* store = it >= 2 ? sv.dinc + (size_t)(it - 2) * cap : nullptr;
      rc = lv_solver_sweep_guess(c, c->s.P, it, D, store);
      if (rc) return rc;
    }
    rc = lv_solver_solve(c, c->s.P, nullptr, it - 1);
    if (rc) return rc;
  }
  if (guess && niter >= 1) {
    KernelTimer kt(c, LV_KF_RHS);
    rc = lv_solver_sweep_store(c, c->s.P, sv.dinc + (size_t)(niter - 1) * cap);
    if (rc) return rc;
    c->sg_valid = niter;
    c->sg_n = c->n;
  }
  if (stats) {
    rc = lv_solver_fetch_stats(c, stats, niter);
    if (rc) return rc;
    return sync_status(c);
  }
  return LV_OK;
}

int lv_export_system(lv_ctx* c, int64_t* nnz, double* diag, int64_t* rowptr, int32_t* col, double* w, double* b) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  if (!c->op_ready) return lv_fail(c, LV_ERR_NOT_MESHED, "the pressure operator has not been assembled");
  const int n = c->n;
  std::vector<int> rp(n + 1);
  cudaMemcpyAsync(rp.data(), c->sv.rowptr, 4 * ((size_t)n + 1), cudaMemcpyDeviceToHost, c->stream);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return lv_cuda_check(c, e, "lv_export_system");
  if (nnz) *nnz = rp[n];
  if (rowptr)
    for (int i = 0; i <= n; ++i) rowptr[i] = rp[i];
  if (diag) cudaMemcpyAsync(diag, c->sv.diag, 8 * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
  if (col) cudaMemcpyAsync(col, c->sv.col, 4 * (size_t)rp[n], cudaMemcpyDeviceToHost, c->stream);
  if (w) cudaMemcpyAsync(w, c->sv.w, 8 * (size_t)rp[n], cudaMemcpyDeviceToHost, c->stream);
  if (b) cudaMemcpyAsync(b, c->sv.b, 8 * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
  e = cudaStreamSynchronize(c->stream);
  return lv_cuda_check(c, e, "lv_export_system");
}

int lv_solve(lv_ctx* c, const double* b, double* x, lv_solve_stats* stats) {
  if (!c || !b || !x) return LV_ERR_BAD_ARGUMENT;
  const size_t n = c->n;
  double* xd = c->sv.xs;
  cudaMemcpyAsync(c->sv.b, b, 8 * n, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(xd, x, 8 * n, cudaMemcpyHostToDevice, c->stream);
  int rc = lv_solver_solve(c, xd, nullptr, 0);
  if (rc) return rc;
  cudaMemcpyAsync(x, xd, 8 * n, cudaMemcpyDeviceToHost, c->stream);
  lv_solve_stats st;
  rc = lv_solver_fetch_stats(c, &st, 1);
  if (rc) return rc;
  if (stats) *stats = st;
  rc = sync_status(c);
  if (rc) return rc;
  return st.converged ? LV_OK : lv_fail(c, LV_ERR_CG_MAXITER, "the solve stopped at itmax above the tolerance");
}

int lv_operator_apply(lv_ctx* c, const double* x, double* y) {
  if (!c || !x || !y) return LV_ERR_BAD_ARGUMENT;
  const size_t n = c->n;
  double* xd = c->sv.xs;
  double* yd = c->sv.q;
  cudaMemcpyAsync(xd, x, 8 * n, cudaMemcpyHostToDevice, c->stream);
  int rc = lv_solver_apply(c, xd, yd);
  if (rc) return rc;
  cudaMemcpyAsync(y, yd, 8 * n, cudaMemcpyDeviceToHost, c->stream);
  return sync_status(c);
}

int lv_multiphase_projection(lv_ctx* c, double quality_threshold, lv_solve_stats* stats) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  Timer t(c, 3);
  return lv_phys_multiphase(c, quality_threshold, stats);
}

int lv_get_timings(lv_ctx* c, double* out, int32_t cap) {
  if (!c || !out) return 0;
  int k = 0;
  for (; k < cap && k < 4; ++k) out[k] = c->t_ms[k];
  return k;
}

int lv_reset_timings(lv_ctx* c) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  for (double& t : c->t_ms) t = 0;
  return LV_OK;
}

int64_t lv_launch_count(const lv_ctx* c) { return c ? c->launches : 0; }

void* lv_stream(lv_ctx* c) { return c ? (void*)c->stream : nullptr; }

int lv_kernel_timing(lv_ctx* c, int32_t enable) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  c->ktiming = enable != 0;
  return LV_OK;
}

int lv_kernel_time(lv_ctx* c, int32_t fam, int64_t* launches, double* ms, int32_t reset) {
  if (!c || fam < 0 || fam >= LV_KF_COUNT) return LV_ERR_BAD_ARGUMENT;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return lv_cuda_check(c, e, "lv_kernel_time");
  auto& k = c->kev[fam];
  double tot = 0.0;
  for (size_t t = 0; t + 1 < k.used; t += 2) {
    float x = 0.0f;
    cudaEventElapsedTime(&x, k.ev[t], k.ev[t + 1]);
    tot += x;
  }
  if (launches) *launches = k.launches;
  if (ms) *ms = tot;
  if (reset) {
    k.used = 0;
    k.launches = 0;
  }
  return LV_OK;
}

int lv_mesh_captures(lv_ctx* c, int32_t* count) {
  if (!c || !count) return LV_ERR_BAD_ARGUMENT;
  if (!c->meshed) return lv_fail(c, LV_ERR_NOT_MESHED, "the grid has not been meshed");
  int v = 0;
  if (int rc = lv_mesh_captures_count(c, &v)) return rc;
  *count = v;
  return LV_OK;
}

int lv_solver_forget(lv_ctx* c) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  c->sg_valid = 0;
  c->sg_pending = false;
  return LV_OK;
}

int lv_solver_halo(lv_ctx* c, int32_t* max_rows) {
  if (!c || !max_rows) return LV_ERR_BAD_ARGUMENT;
  int m = 0;
  if (int rc = lv_fcg_halo_info(c, &m)) return rc;
  *max_rows = m;
  return LV_OK;
}

int lv_set_wait_limit(lv_ctx* c, int64_t cycles) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  c->spin_limit = cycles > 0 ? (long long)cycles : LV_WAIT_LIMIT_DEFAULT;
  return LV_OK;
}

int lv_solver_unconverged(lv_ctx* c, int64_t* solves) {
  if (!c || !solves) return LV_ERR_BAD_ARGUMENT;
  long long h[3] = {0, 0, 0};
  cudaMemcpyAsync(h, c->sv.counters, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return lv_cuda_check(c, e, "lv_solver_unconverged");
  *solves = h[2];
  return LV_OK;
}

int lv_solver_counters(lv_ctx* c, int64_t* solves, int64_t* iterations) {
  if (!c) return LV_ERR_BAD_ARGUMENT;
  long long h[2] = {0, 0};
  cudaMemcpyAsync(h, c->sv.counters, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return lv_cuda_check(c, e, "lv_solver_counters");
  if (solves) *solves = h[0];
  if (iterations) *iterations = h[1];
  return LV_OK;
}

}  // extern "C"
