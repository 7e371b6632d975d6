// lvref — CPU oracle for the Lagrangian Voronoi per-timestep path.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, in plain C++ FP64, the
// algorithms of LagrangianVoronoi.jl (Julia, v0.1.0) that the GPU library
// replaces.  Only the tests, the smoke check and the CPU-baseline leg of the
// benchmark load it; the product library never links or calls it.
//
// Faithfulness rules followed throughout:
//  * every floating-point expression keeps the reference's evaluation order
//    (Julia evaluates a*b/c*d left to right, SVector ops elementwise) and the
//    file is compiled with -ffp-contract=off so no multiply-add is fused;
//  * seeds are inserted into the cell list in index order, which is what the
//    reference does when run with one thread (julia -t 1);
//  * neighbour labels are 0-based particle indices; boundary labels keep the
//    reference's values BDARY_UP/RIGHT/DOWN/LEFT = -1/-2/-3/-4
//    (src/polygon.jl:4-7), so "label < 0" is the reference's "label <= 0".
//
// Third-party arithmetic: Krylov.jl 0.9.8 `minres!` (Manifest.toml:465-469)
// is not vendored with the reference; `minres_solve` below restates MINRES from
// Paige & Saunders (1975) with Krylov.jl's documented stopping rule
// ||r|| <= atol + rtol*||r0||.  StaticArrays `norm` is restated as
// sqrt(x1^2 + x2^2).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double SIGNUM_EPS = 2.0 * 2.220446049250313e-16;  // polygon.jl:2
constexpr int64_t BDARY_UP = -1, BDARY_RIGHT = -2, BDARY_DOWN = -3, BDARY_LEFT = -4;

struct V2 {
  double x, y;
};
inline V2 operator+(V2 a, V2 b) { return {a.x + b.x, a.y + b.y}; }
inline V2 operator-(V2 a, V2 b) { return {a.x - b.x, a.y - b.y}; }
inline V2 operator*(double s, V2 a) { return {s * a.x, s * a.y}; }
inline double dot(V2 a, V2 b) { return a.x * b.x + a.y * b.y; }
inline double cross2(V2 a, V2 b) { return a.x * b.y - a.y * b.x; }  // geometry.jl:72-74
inline double norm_squared(V2 a) { return dot(a, a); }
inline double norm(V2 a) { return std::sqrt(a.x * a.x + a.y * a.y); }
inline bool veq(V2 a, V2 b) { return a.x == b.x && a.y == b.y; }

struct M2 {  // column-major like RealMatrix (geometry.jl:13)
  double a11, a21, a12, a22;
};

struct Edge {  // geometry.jl:82-87
  V2 v1, v2;
  int64_t label;
};

inline int signum(double x) {  // polygon.jl:9-16
  if (x < -SIGNUM_EPS) return -1;
  if (x > SIGNUM_EPS) return 1;
  return 0;
}

inline double jmax(double a, double b) { return (b > a) ? b : a; }
inline double jmin(double a, double b) { return (b < a) ? b : a; }

enum Status {
  ST_OK = 0,
  ST_NAN_VELOCITY = 1,
  ST_MESH_DESTROYED = 2,
  ST_EDGE_OVERFLOW = 3,
  ST_BAD_ARGUMENT = 6,
  ST_NONFINITE_POSITION = 10,
};

struct PathNode {
  int64_t i1, i2;
  int64_t keysq;
  double rr;
};

struct Grid {
  // geometry of the domain (voronoigrid.jl:14-50)
  V2 bmin, bmax, cmin, cmax;
  double dr, h, r_max, rr_max, xperiod, yperiod;
  bool xper, yper;
  // cell list (neighborlist.jl:11-44)
  V2 origin;
  int64_t n1, n2;
  std::vector<PathNode> path;
  std::vector<std::vector<int32_t>> cells;
  // particles, SoA
  int n = 0;
  std::vector<V2> x, v, dv, momentum;
  std::vector<double> rho, e, P, c2, mass, energy, quality, mu;
  std::vector<double> T, kc, cV;  // PolygonNSF (celldefs.jl:49-56): temperature, conductivity, specific heat
  std::vector<int32_t> phase;
  std::vector<M2> D;
  std::vector<std::vector<Edge>> edges;
  int max_edges = 64;
  // pressure operator and solver (pressure.jl:89-159)
  std::vector<double> diag;
  std::vector<std::vector<int32_t>> op_nbr;
  std::vector<std::vector<double>> op_w;
  std::vector<double> b, Psol;
  // the change of each find_pressure sweep in the last call with the GPU
  // solver's initial guess (method 2), stored in FP32 as the GPU does
  std::vector<std::vector<double>> sweep_inc;
  int sweep_n = 0;
  std::vector<V2> GP;
  int status = ST_OK;
  // boundary closures evaluated per boundary edge by the caller (the order of
  // boundaries(p) over the polygons, iterators.jl:46-57): velocity and
  // charfun flag; used instead of the label table while edge_mode is set
  bool edge_mode = false;
  std::vector<V2> edge_vel;
  std::vector<uint8_t> edge_act;
};

// first boundary edge of every polygon in the per-edge order
std::vector<int64_t> boundary_offsets(const Grid& g) {
  std::vector<int64_t> off(g.n + 1, 0);
  for (int i = 0; i < g.n; ++i) {
    int64_t c = 0;
    for (const auto& e : g.edges[i]) c += e.label < 0 ? 1 : 0;
    off[i + 1] = off[i] + c;
  }
  return off;
}

// ---------------------------------------------------------------- cell list

// neighborlist.jl:29-41 — the path of cell offsets visited by the candidate
// search.  The reference builds the full (2n-1)^2 path; only the prefix with
// rr <= rr_max plus the first node beyond it can ever be visited (the loop
// either breaks there or throws), so only that prefix is built.  The offset
// ranges keep the reference's swap of n1/n2 (neighborlist.jl:30-31).
void build_path(Grid& g) {
  g.path.clear();
  const int64_t R = (int64_t)std::ceil(std::sqrt(g.rr_max) / g.h) + 3;
  const int64_t lo2 = std::max<int64_t>(1 - g.n1, -R), hi2 = std::min<int64_t>(g.n1 - 1, R);
  const int64_t lo1 = std::max<int64_t>(1 - g.n2, -R), hi1 = std::min<int64_t>(g.n2 - 1, R);
  std::vector<PathNode> all;
  for (int64_t i2 = lo2; i2 <= hi2; ++i2)
    for (int64_t i1 = lo1; i1 <= hi1; ++i1) {
      int64_t a = std::max<int64_t>(0, std::llabs(i1) - 1), c = std::max<int64_t>(0, std::llabs(i2) - 1);
      double rr = (g.h * g.h) * (double)(a * a + c * c);
      all.push_back({i1, i2, i1 * i1 + i2 * i2, rr});
    }
  // sort!(by = |key|^2) then sort!(by = rr), both stable.
  std::stable_sort(all.begin(), all.end(), [](const PathNode& p, const PathNode& q) { return p.keysq < q.keysq; });
  std::stable_sort(all.begin(), all.end(), [](const PathNode& p, const PathNode& q) { return p.rr < q.rr; });
  for (const auto& nd : all) {
    g.path.push_back(nd);
    if (nd.rr > g.rr_max) break;
  }
}

// neighborlist.jl:47-52
inline bool findkey(const Grid& g, V2 x, int64_t& i1, int64_t& i2) {
  V2 d = x - g.origin;
  double f1 = std::floor(d.x / g.h), f2 = std::floor(d.y / g.h);
  if (!std::isfinite(f1) || !std::isfinite(f2) || std::fabs(f1) > 4e18 || std::fabs(f2) > 4e18) return false;
  i1 = (int64_t)f1 + 1;
  i2 = (int64_t)f2 + 1;
  return true;
}

// neighborlist.jl:55-67
inline void cl_insert(Grid& g, V2 x, int32_t label) {
  int64_t i1, i2;
  if (!findkey(g, x, i1, i2)) {
    g.status = ST_NONFINITE_POSITION;
    return;
  }
  if (i1 >= 1 && i1 <= g.n1 && i2 >= 1 && i2 <= g.n2) g.cells[(i1 - 1) + g.n1 * (i2 - 1)].push_back(label);
}

// voronoigrid.jl:130-147
void insert_periodic(Grid& g, V2 x, int32_t label) {
  V2 X{g.xperiod, 0.0}, Y{0.0, g.yperiod};
  cl_insert(g, x, label);
  if (g.xper) {
    cl_insert(g, x + X, label);
    cl_insert(g, x - X, label);
  }
  if (g.yper) {
    cl_insert(g, x + Y, label);
    cl_insert(g, x - Y, label);
  }
  if (g.xper && g.yper) {
    cl_insert(g, (x + X) + Y, label);
    cl_insert(g, (x + X) - Y, label);
    cl_insert(g, (x - X) + Y, label);
    cl_insert(g, (x - X) - Y, label);
  }
}

// voronoigrid.jl:116-125
inline V2 get_arrow(const Grid& g, V2 a, V2 b) {
  V2 v = a - b;
  if (g.xper && std::fabs(v.x) > 0.5 * g.xperiod) v.x -= (v.x > 0 ? 1.0 : -1.0) * g.xperiod;
  if (g.yper && std::fabs(v.y) > 0.5 * g.yperiod) v.y -= (v.y > 0 ? 1.0 : -1.0) * g.yperiod;
  return v;
}

// ------------------------------------------------------------------ polygon

// polygon.jl:37-47
void reset_poly(const Grid& g, std::vector<Edge>& E) {
  E.clear();
  V2 A = g.cmin, C = g.cmax, B{C.x, A.y}, D{A.x, C.y};
  E.push_back({B, A, BDARY_DOWN});
  E.push_back({A, D, BDARY_LEFT});
  E.push_back({D, C, BDARY_UP});
  E.push_back({C, B, BDARY_RIGHT});
}

// polygon.jl:101-107
double influence_rr(const std::vector<Edge>& E, V2 x) {
  double rr = 0.0;
  for (const auto& e : E) rr = jmax(rr, 4.0 * norm_squared(e.v1 - x));
  return rr;
}

// polygon.jl:51-97 — half-plane clip; deletion swaps in the last edge
// (fastvector.jl:44-50).  Returns 1 on a cut, 0 otherwise, -1 on overflow.
int voronoicut_poly(std::vector<Edge>& E, V2 px, V2 y, int64_t label, int max_edges) {
  V2 diff = y - px;
  V2 mid = 0.5 * (y + px);
  double c = dot(diff, mid);
  const double qnan = std::numeric_limits<double>::quiet_NaN();
  V2 X{qnan, qnan}, Y{qnan, qnan};
  size_t i = 0;
  while (i < E.size()) {
    Edge e = E[i];
    double f1 = dot(diff, e.v1) - c;
    double f2 = dot(diff, e.v2) - c;
    int s1 = signum(f1), s2 = signum(f2);
    int s12 = s1 + s2;
    if (0 <= s12 && s12 <= 1 && (s1 | s2) != 0) {
      Y = X;
      double inv = 1.0 / (f1 - f2);
      V2 t{f1 * e.v2.x - f2 * e.v1.x, f1 * e.v2.y - f2 * e.v1.y};
      X = V2{inv * t.x, inv * t.y};
      if (s1 == 0) X = e.v1;
      if (s2 == 0) X = e.v2;
      E[i] = (s1 == 1) ? Edge{X, e.v2, e.label} : Edge{e.v1, X, e.label};
    }
    if (1 <= s12) {
      if (E.size() - 1 > i) E[i] = E.back();
      E.pop_back();
    } else {
      ++i;
    }
  }
  bool ynull = std::isnan(Y.x) && std::isnan(Y.y);
  if (!ynull && !veq(X, Y)) {
    Edge ne{X, Y, label};
    if (cross2(Y - X, px - X) > 0.0) ne = Edge{Y, X, label};
    if ((int)E.size() >= max_edges) return -1;
    E.push_back(ne);
    return 1;
  }
  return 0;
}

// IO.jl:35-48
void sort_edges(std::vector<Edge>& E) {
  const size_t n = E.size();
  for (size_t i = 0; i < n; ++i) {
    V2 last = E[i].v2;
    for (size_t j = i + 1; j < n; ++j) {
      if (veq(last, E[j].v1)) {
        std::swap(E[i + 1], E[j]);
        break;
      }
    }
  }
}

// polygon.jl:114-121
double poly_area(const std::vector<Edge>& E, V2 x) {
  double A = 0.0;
  for (const auto& e : E) A += 0.5 * std::fabs(cross2(e.v1 - x, e.v2 - x));
  return A;
}

// polygon.jl:201-219
V2 poly_centroid(const std::vector<Edge>& E, V2 x) {
  double A = 0.0;
  V2 c{0.0, 0.0};
  for (const auto& e : E) {
    double dA = 0.5 * std::fabs(cross2(e.v1 - x, e.v2 - x));
    A += dA;
    V2 s = (x + e.v1) + e.v2;
    c = c + V2{(dA * s.x) / 3.0, (dA * s.y) / 3.0};
  }
  return V2{c.x / A, c.y / A};
}

// polygon.jl:228-232
inline double lr_ratio(V2 dx, const Edge& e) {
  double l2 = norm_squared(e.v1 - e.v2);
  double r2 = norm_squared(dx);
  return std::sqrt(l2 / r2);
}
inline V2 midpoint(const Edge& e) { return 0.5 * (e.v1 + e.v2); }  // geometry.jl:145-147
inline double len(const Edge& e) { return norm(e.v1 - e.v2); }     // geometry.jl:136-138
inline V2 normal_vector(const Edge& e) {                            // polygon.jl:153-156
  V2 n{e.v1.y - e.v2.y, e.v2.x - e.v1.x};
  double nn = norm(n);
  return V2{n.x / nn, n.y / nn};
}

// voronoigrid.jl:53-81 — candidate loop for one polygon.
int voronoicut_grid(const Grid& g, int i, std::vector<Edge>& E) {
  V2 x = g.x[i];
  double prr = influence_rr(E, x);
  int64_t k1, k2;
  if (!findkey(g, x, k1, k2)) return ST_NONFINITE_POSITION;
  for (const auto& nd : g.path) {
    if (nd.rr > prr) break;
    if (nd.rr > g.rr_max) return ST_MESH_DESTROYED;
    int64_t c1 = k1 + nd.i1, c2 = k2 + nd.i2;
    if (c1 < 1 || c1 > g.n1 || c2 < 1 || c2 > g.n2) continue;
    for (int32_t j : g.cells[(c1 - 1) + g.n1 * (c2 - 1)]) {
      V2 y = x + get_arrow(g, g.x[j], x);
      if (veq(x, y) || norm_squared(x - y) > prr) continue;
      int r = voronoicut_poly(E, x, y, j, g.max_edges);
      if (r < 0) return ST_EDGE_OVERFLOW;
      if (r) prr = influence_rr(E, x);
    }
  }
  return ST_OK;
}

// voronoigrid.jl:89-108
int remesh(Grid& g) {
  g.status = ST_OK;
  for (auto& c : g.cells) c.clear();
  g.edges.resize(g.n);
  for (int i = 0; i < g.n; ++i) {
    reset_poly(g, g.edges[i]);
    insert_periodic(g, g.x[i], i);
  }
  if (g.status != ST_OK) return g.status;
  int worst = ST_OK;
#pragma omp parallel for schedule(dynamic, 64) reduction(max : worst)
  for (int i = 0; i < g.n; ++i) {
    int st = voronoicut_grid(g, i, g.edges[i]);
    sort_edges(g.edges[i]);
    worst = std::max(worst, st);
  }
  g.status = worst;
  return worst;
}

// ------------------------------------------------------------ face iterator

// iterators.jl:23-33: interior faces (q, e, y) of polygon i.
template <class F>
inline void for_faces(const Grid& g, int i, F&& f) {
  const V2 x = g.x[i];
  for (const auto& e : g.edges[i]) {
    if (e.label < 0) continue;
    int j = (int)e.label;
    V2 y = x + get_arrow(g, g.x[j], x);
    f(j, e, y);
  }
}

// ------------------------------------------------------------ physics steps

inline double eint(const Grid& g, int i) {  // pressure.jl:32-34
  return g.e[i] - 0.5 * norm_squared(g.v[i]);
}

void ideal_eos(Grid& g, double gamma, double Pmin) {  // pressure.jl:49-55
#pragma omp parallel for
  for (int i = 0; i < g.n; ++i) {
    g.rho[i] = g.mass[i] / poly_area(g.edges[i], g.x[i]);
    g.P[i] = (gamma - 1.0) * g.rho[i] * eint(g, i);
    g.c2[i] = gamma * jmax(g.P[i], Pmin) / g.rho[i];
  }
}

void stiffened_eos(Grid& g, double gamma, double P0) {  // pressure.jl:64-70
#pragma omp parallel for
  for (int i = 0; i < g.n; ++i) {
    g.rho[i] = g.mass[i] / poly_area(g.edges[i], g.x[i]);
    g.P[i] = (gamma - 1.0) * g.rho[i] * eint(g, i);
    g.c2[i] = gamma * (g.P[i] + P0) / g.rho[i];
  }
}

void find_rho(Grid& g) {  // pressure.jl:36-40
#pragma omp parallel for
  for (int i = 0; i < g.n; ++i) g.rho[i] = g.mass[i] / poly_area(g.edges[i], g.x[i]);
}

void gravity_step(Grid& g, V2 gv, double dt) {  // pressure.jl:77-82
#pragma omp parallel for
  for (int i = 0; i < g.n; ++i) g.v[i] = g.v[i] + dt * gv;
}

void pressure_step(Grid& g, double dt) {  // pressure.jl:10-25
#pragma omp parallel for
  for (int i = 0; i < g.n; ++i) {
    V2 vi = g.v[i];
    const V2 xi = g.x[i];
    for_faces(g, i, [&](int j, const Edge& e, V2 y) {
      double lrr = lr_ratio(xi - y, e);
      V2 m = midpoint(e);
      double s = dt / g.mass[i] * lrr * (g.P[i] - g.P[j]);
      vi = vi + s * (m - xi);
    });
    g.v[i] = vi;
  }
#pragma omp parallel for
  for (int i = 0; i < g.n; ++i) {
    double ei = g.e[i];
    const V2 xi = g.x[i];
    for_faces(g, i, [&](int j, const Edge& e, V2 y) {
      double lrr = lr_ratio(xi - y, e);
      V2 m = midpoint(e);
      ei -= dt * lrr / g.mass[i] * (dot(m - xi, g.P[i] * g.v[i]) - dot(m - y, g.P[j] * g.v[j]));
    });
    g.e[i] = ei;
  }
}

// pressure.jl:104-117
void refresh_operator(Grid& g, double dt) {
  g.diag.assign(g.n, 0.0);
  g.op_nbr.assign(g.n, {});
  g.op_w.assign(g.n, {});
#pragma omp parallel for
  for (int i = 0; i < g.n; ++i) {
    g.diag[i] = g.mass[i] / (g.rho[i] * g.rho[i] * g.c2[i] * (dt * dt));
    const V2 xi = g.x[i];
    for_faces(g, i, [&](int j, const Edge& e, V2 y) {
      g.op_nbr[i].push_back(j);
      g.op_w[i].push_back(lr_ratio(xi - y, e) * (0.5 / g.rho[i] + 0.5 / g.rho[j]));
    });
  }
}

// pressure.jl:119-130
void op_mul(const Grid& g, const double* xin, double* y) {
#pragma omp parallel for
  for (int i = 0; i < g.n; ++i) {
    double yi = g.diag[i] * xin[i];
    for (size_t k = 0; k < g.op_nbr[i].size(); ++k) yi += g.op_w[i][k] * (xin[i] - xin[g.op_nbr[i][k]]);
    y[i] = yi;
  }
}

// Deterministic blocked dot product (independent of the thread count).
double bdot(const double* a, const double* b, int n) {
  const int B = 4096;
  int nb = (n + B - 1) / B;
  std::vector<double> part(nb, 0.0);
#pragma omp parallel for
  for (int k = 0; k < nb; ++k) {
    double s = 0.0;
    int hi = std::min(n, (k + 1) * B);
    for (int i = k * B; i < hi; ++i) s += a[i] * b[i];
    part[k] = s;
  }
  double s = 0.0;
  for (double p : part) s += p;
  return s;
}

// pressure.jl:162-203 — right-hand side, warm start and pressure gradient.
// vbc[4][2] holds a constant wall velocity per boundary label (-1..-4).
void refresh_rhs(Grid& g, double dt, bool gp_step, const double* vbc) {
  const std::vector<int64_t> boff = g.edge_mode ? boundary_offsets(g) : std::vector<int64_t>();
  g.b.assign(g.n, 0.0);
  g.Psol.assign(g.n, 0.0);
  g.GP.assign(g.n, V2{0.0, 0.0});
#pragma omp parallel for
  for (int i = 0; i < g.n; ++i) {
    const V2 xi = g.x[i];
    double A = poly_area(g.edges[i], xi);
    double bi = A * g.P[i] / (g.rho[i] * g.c2[i] * (dt * dt));
    g.Psol[i] = g.P[i];
    V2 gp{0.0, 0.0};
    for_faces(g, i, [&](int j, const Edge& e, V2 y) {
      double lrr = lr_ratio(xi - y, e);
      V2 m = midpoint(e);
      bi -= (lrr / dt) * dot(g.v[i] - g.v[j], m - y);
      gp = gp - (lrr * (g.P[i] - g.P[j])) * (m - xi);
    });
    int64_t q = g.edge_mode ? boff[i] : 0;
    for (const auto& e : g.edges[i]) {
      if (e.label >= 0) continue;
      V2 dS{e.v1.y - e.v2.y, e.v2.x - e.v1.x};
      int slot = (int)(-e.label - 1);
      // vbc = boundary_velocity(midpoint(e), e.label) (pressure.jl:182)
      V2 wall = g.edge_mode ? g.edge_vel[q++] : (vbc ? V2{vbc[2 * slot], vbc[2 * slot + 1]} : V2{0.0, 0.0});
      bi -= dot(dS, wall - g.v[i]) / dt;
    }
    g.b[i] = bi;
    g.GP[i] = V2{gp.x / g.mass[i], gp.y / g.mass[i]};
  }
  if (gp_step) {
#pragma omp parallel for
    for (int i = 0; i < g.n; ++i) {
      const V2 xi = g.x[i];
      double bi = g.b[i];
      for_faces(g, i, [&](int j, const Edge& e, V2 y) {
        double lrr = lr_ratio(xi - y, e);
        V2 m = midpoint(e);
        V2 z = 0.5 * (xi + y);
        bi += lrr * dot(g.GP[i] - g.GP[j], m - z);
      });
      g.b[i] = bi;
    }
  }
}

struct SolveStats {
  int32_t iterations;
  int32_t converged;
  double rel_residual;  // ||b - A x|| / ||b|| recomputed at exit
};

// MINRES (Paige & Saunders 1975) with warm start; stops when
// ||r|| <= atol + rtol*||r0|| or when the least-squares test
// ||A r|| <= rtol*||A||*||r|| holds (inconsistent singular systems).
template <class Op>
int minres_op(int n, Op op_apply, const std::vector<double>& bvec, std::vector<double>& x, double atol, double rtol,
              int itmax, SolveStats* st);

int minres_solve(const Grid& g, const std::vector<double>& bvec, std::vector<double>& x, double atol, double rtol,
                 int itmax, SolveStats* st) {
  return minres_op(g.n, [&](const double* in, double* out) { op_mul(g, in, out); }, bvec, x, atol, rtol, itmax, st);
}

// The same MINRES with the operator y = A x given by op_apply(x, y) on n unknowns.
template <class Op>
int minres_op(int n, Op op_apply, const std::vector<double>& bvec, std::vector<double>& x, double atol, double rtol,
              int itmax, SolveStats* st) {
  std::vector<double> r1(n), r2(n), y(n), v(n), w(n, 0.0), w1(n), w2(n, 0.0), Ax(n);
  op_apply(x.data(), Ax.data());
  for (int i = 0; i < n; ++i) r1[i] = bvec[i] - Ax[i];
  y = r1;
  double beta1 = std::sqrt(bdot(r1.data(), y.data(), n));
  int itn = 0;
  bool solved = (beta1 == 0.0);
  if (!solved) {
    r2 = r1;
    double oldb = 0.0, beta = beta1, dbar = 0.0, epsln = 0.0, phibar = beta1;
    double cs = -1.0, sn = 0.0, tnorm2 = 0.0;
    const double eps = std::numeric_limits<double>::epsilon();
    double tol = atol + rtol * beta1;
    while (itn < itmax) {
      ++itn;
      double s = 1.0 / beta;
      for (int i = 0; i < n; ++i) v[i] = s * y[i];
      op_apply(v.data(), y.data());
      if (itn >= 2)
        for (int i = 0; i < n; ++i) y[i] -= (beta / oldb) * r1[i];
      double alfa = bdot(v.data(), y.data(), n);
      for (int i = 0; i < n; ++i) y[i] -= (alfa / beta) * r2[i];
      r1.swap(r2);
      r2 = y;
      oldb = beta;
      beta = std::sqrt(bdot(r2.data(), y.data(), n));
      tnorm2 += alfa * alfa + oldb * oldb + beta * beta;
      double oldeps = epsln;
      double delta = cs * dbar + sn * alfa;
      double gbar = sn * dbar - cs * alfa;
      epsln = sn * beta;
      dbar = -cs * beta;
      double root = std::sqrt(gbar * gbar + dbar * dbar);
      double gamma = std::max(std::sqrt(gbar * gbar + beta * beta), eps);
      cs = gbar / gamma;
      sn = beta / gamma;
      double phi = cs * phibar;
      phibar = sn * phibar;
      double denom = 1.0 / gamma;
      w1.swap(w2);
      w2.swap(w);
      for (int i = 0; i < n; ++i) {
        w[i] = (v[i] - oldeps * w1[i] - delta * w2[i]) * denom;
        x[i] += phi * w[i];
      }
      double rnorm = phibar;
      double Anorm = std::sqrt(tnorm2);
      double Arnorm = phibar * root;
      if (rnorm <= tol) {
        solved = true;
        break;
      }
      if (Anorm > 0 && rnorm > 0 && Arnorm / (Anorm * rnorm) <= rtol) {
        solved = true;
        break;
      }
      if (beta == 0.0) {
        solved = true;
        break;
      }
    }
  }
  if (st) {
    op_apply(x.data(), Ax.data());
    std::vector<double> r(n);
    for (int i = 0; i < n; ++i) r[i] = bvec[i] - Ax[i];
    double bn = std::sqrt(bdot(bvec.data(), bvec.data(), n));
    double rn = std::sqrt(bdot(r.data(), r.data(), n));
    st->iterations = itn;
    st->converged = solved ? 1 : 0;
    st->rel_residual = bn > 0 ? rn / bn : rn;
  }
  return ST_OK;
}

// Jacobi-preconditioned CG on the same operator (the GPU solver's algorithm).
// If every diagonal term vanishes (c2 = Inf everywhere) the operator is a graph
// Laplacian with the constants as null space: b is projected to zero mean.
// Stops when ||r|| <= tol*||b|| (recursive residual) or after itmax iterations.
int pcg_solve(const Grid& g, std::vector<double> bvec, std::vector<double>& x, double tol, int itmax,
              SolveStats* st) {
  const int n = g.n;
  bool singular = true;
  for (int i = 0; i < n; ++i)
    if (g.diag[i] != 0.0) {
      singular = false;
      break;
    }
  if (singular && n > 0) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += bvec[i];
    double mean = s / n;
    for (int i = 0; i < n; ++i) bvec[i] -= mean;
  }
  std::vector<double> Adiag(n), r(n), z(n), p(n), q(n);
  for (int i = 0; i < n; ++i) {
    double s = g.diag[i];
    for (double w : g.op_w[i]) s += w;
    Adiag[i] = s;
  }
  op_mul(g, x.data(), q.data());
  for (int i = 0; i < n; ++i) {
    r[i] = bvec[i] - q[i];
    z[i] = r[i] / Adiag[i];
    p[i] = z[i];
  }
  double rz = bdot(r.data(), z.data(), n);
  double bnorm = std::sqrt(bdot(bvec.data(), bvec.data(), n));
  double rnorm = std::sqrt(bdot(r.data(), r.data(), n));
  int it = 0;
  while (rnorm > tol * bnorm && it < itmax) {
    op_mul(g, p.data(), q.data());
    double alpha = rz / bdot(p.data(), q.data(), n);
    for (int i = 0; i < n; ++i) {
      x[i] += alpha * p[i];
      r[i] -= alpha * q[i];
      z[i] = r[i] / Adiag[i];
    }
    double rz_new = bdot(r.data(), z.data(), n);
    rnorm = std::sqrt(bdot(r.data(), r.data(), n));
    double beta = rz_new / rz;
    rz = rz_new;
    for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    ++it;
  }
  if (st) {
    op_mul(g, x.data(), q.data());
    double rn2 = 0.0;
    for (int i = 0; i < n; ++i) r[i] = bvec[i] - q[i];
    rn2 = bdot(r.data(), r.data(), n);
    st->iterations = it;
    st->converged = (rnorm <= tol * bnorm) ? 1 : 0;
    st->rel_residual = bnorm > 0 ? std::sqrt(rn2) / bnorm : std::sqrt(rn2);
  }
  return ST_OK;
}

void viscous_step(Grid& g, double dt, bool artificial_viscosity) {  // diffusion.jl:39-53
  const double avdr = artificial_viscosity ? g.dr : 0.0;
  std::vector<M2> S(g.n);
  // diffusion.jl:22-29 getS
#pragma omp parallel for
  for (int i = 0; i < g.n; ++i) {
    const M2 D = g.D[i];
    double divv = D.a11 + D.a22;
    double mu = g.mu[i];
    if (divv < 0.0) mu -= divv * g.rho[i] * (avdr * avdr);
    double c = 2.0 * mu;
    S[i] = M2{c * (D.a11 - divv / 3.0), c * D.a21, c * D.a12, c * (D.a22 - divv / 3.0)};
  }
#pragma omp parallel for
  for (int i = 0; i < g.n; ++i) {
    V2 vi = g.v[i];
    const V2 xi = g.x[i];
    for_faces(g, i, [&](int j, const Edge& e, V2 y) {
      V2 m = midpoint(e);
      double c = dt * lr_ratio(xi - y, e) / g.mass[i];
      M2 M{c * (S[i].a11 - S[j].a11), c * (S[i].a21 - S[j].a21), c * (S[i].a12 - S[j].a12),
           c * (S[i].a22 - S[j].a22)};
      V2 d = m - xi;
      vi = vi - V2{M.a11 * d.x + M.a12 * d.y, M.a21 * d.x + M.a22 * d.y};
    });
    g.v[i] = vi;
  }
#pragma omp parallel for
  for (int i = 0; i < g.n; ++i) {
    double ei = g.e[i];
    const V2 xi = g.x[i];
    const M2 Si = S[i];
    V2 Sv{Si.a11 * g.v[i].x + Si.a12 * g.v[i].y, Si.a21 * g.v[i].x + Si.a22 * g.v[i].y};
    for_faces(g, i, [&](int j, const Edge& e, V2 y) {
      V2 m = midpoint(e);
      const M2 Sj = S[j];
      V2 Sqv{Sj.a11 * g.v[j].x + Sj.a12 * g.v[j].y, Sj.a21 * g.v[j].x + Sj.a22 * g.v[j].y};
      ei += dt * lr_ratio(xi - y, e) / g.mass[i] * (dot(m - xi, Sv) - dot(m - y, Sqv));
    });
    g.e[i] = ei;
  }
}

void find_D(Grid& g) {  // diffusion.jl:8-19
#pragma omp parallel for
  for (int i = 0; i < g.n; ++i) {
    M2 D{0.0, 0.0, 0.0, 0.0};
    const V2 xi = g.x[i];
    for_faces(g, i, [&](int j, const Edge& e, V2 y) {
      V2 m = midpoint(e);
      double lrr = lr_ratio(xi - y, e);
      V2 a = g.v[i] - g.v[j], b = m - y;
      D.a11 += lrr * (a.x * b.x);
      D.a21 += lrr * (a.y * b.x);
      D.a12 += lrr * (a.x * b.y);
      D.a22 += lrr * (a.y * b.y);
    });
    double A = poly_area(g.edges[i], xi);
    D = M2{D.a11 / A, D.a21 / A, D.a12 / A, D.a22 / A};
    g.D[i] = M2{0.5 * (D.a11 + D.a11), 0.5 * (D.a21 + D.a12), 0.5 * (D.a12 + D.a21), 0.5 * (D.a22 + D.a22)};
  }
}

// diffusion.jl:64-79 with a constant wall velocity per boundary label.
void bdary_friction(Grid& g, const double* vwall, double dt) {
  const std::vector<int64_t> boff = g.edge_mode ? boundary_offsets(g) : std::vector<int64_t>();
#pragma omp parallel for
  for (int i = 0; i < g.n; ++i) {
    double tmp = 1.0;
    V2 vi = g.v[i];
    double ei = g.e[i];
    int64_t q = g.edge_mode ? boff[i] : 0;
    for (const auto& e : g.edges[i]) {
      if (e.label >= 0) continue;
      V2 m = 0.5 * (e.v1 + e.v2);
      const int64_t qe = q++;
      if (g.edge_mode && !g.edge_act.empty() && !g.edge_act[qe]) continue;  // if !charfun(m) continue end
      V2 nv = normal_vector(e);
      double lrr = len(e) / std::fabs(dot(m - g.x[i], nv));
      int slot = (int)(-e.label - 1);
      // vDirichlet(m): per edge, or the label table
      V2 wall = g.edge_mode ? g.edge_vel[qe] : V2{vwall[2 * slot], vwall[2 * slot + 1]};
      V2 f{g.mu[i] * lrr * wall.x / g.mass[i], g.mu[i] * lrr * wall.y / g.mass[i]};
      tmp += dt * g.mu[i] * lrr / g.mass[i];
      ei += dt * dot(f, vi);
      vi = vi + dt * f;
    }
    g.v[i] = V2{vi.x / tmp, vi.y / tmp};
    g.e[i] = ei;
  }
}

// ideal_temperature! (fourier.jl:1-12): T = eint(p)/cV, eint = e - norm_squared(v)/2 (pressure.jl:32-34)
void ideal_temperature(Grid& g) {
#pragma omp parallel for
  for (int i = 0; i < g.n; ++i) g.T[i] = (g.e[i] - 0.5 * dot(g.v[i], g.v[i])) / g.cV[i];
}

// fourier_step! (fourier.jl:14-28)
void fourier_step(Grid& g, double dt) {
#pragma omp parallel for
  for (int i = 0; i < g.n; ++i) {
    const V2 xi = g.x[i];
    double ei = g.e[i];
    for_faces(g, i, [&](int j, const Edge& e, V2 y) {
      double lrr = lr_ratio(xi - y, e);
      double k = 0.5 * (g.kc[i] + g.kc[j]);
      ei = ei - dt * k / g.mass[i] * lrr * (g.T[i] - g.T[j]);
    });
    g.e[i] = ei;
  }
}

// heat_from_bdary! (fourier.jl:30-62) with the wall temperatures T_bc(m,
// label) given per boundary edge in the per-edge order (NaN: adiabatic).
// Returns ST_BAD_ARGUMENT where the reference's @assert(p.cV > 0) fails.
int heat_from_bdary(Grid& g, double dt, const double* Tb) {
  const std::vector<int64_t> boff = boundary_offsets(g);
  int bad = 0;
#pragma omp parallel for reduction(| : bad)
  for (int i = 0; i < g.n; ++i) {
    bool bd = false;
    for (const auto& e : g.edges[i]) bd = bd || e.label < 0;
    if (!bd) continue;
    if (!(g.cV[i] > 0.0)) {
      bad = 1;
      continue;
    }
    double implicit_factor = 1.0;
    const double thermal_D = g.kc[i] / (g.rho[i] * g.cV[i]);
    const double e_kinetic = 0.5 * dot(g.v[i], g.v[i]);
    double T = (g.e[i] - e_kinetic) / g.cV[i];
    const double A = poly_area(g.edges[i], g.x[i]);
    int64_t q = boff[i];
    for (const auto& e : g.edges[i]) {
      if (e.label >= 0) continue;
      const double Tw = Tb[q++];
      V2 m = 0.5 * (e.v1 + e.v2);
      V2 nv = normal_vector(e);
      double lrr = len(e) / std::fabs(dot(m - g.x[i], nv)) + 0.01 * g.dr;
      if (!std::isnan(Tw)) {
        double tmp = dt * thermal_D * lrr / A;
        T += tmp * Tw;
        implicit_factor += tmp;
      }
    }
    T /= implicit_factor;
    g.T[i] = T;
    g.e[i] = e_kinetic + g.cV[i] * T;
  }
  return bad ? ST_BAD_ARGUMENT : ST_OK;
}

// ViscousSolver + viscous_step!(solver, dt) (viscous_solver.jl:43-129): rows
// 2i, 2i+1 (v_index) hold the neighbours' entries -0.5 lrr (mu_i + mu_j) in
// face order, then the self entry vv = m/dt minus them; the ThreadedMat
// product accumulates a row from 0.0 in that order.  MINRES (atol = rtol =
// 1e-6, itmax = 2000) from the first guess v; then v = the solution.
int viscous_solve(Grid& g, double dt, double tol, int itmax, SolveStats* st) {
  const int n = g.n;
  std::vector<std::vector<int32_t>> rows(n);
  std::vector<std::vector<double>> vals(n);
  std::vector<double> b(2 * n), u(2 * n);
#pragma omp parallel for
  for (int i = 0; i < n; ++i) {
    const V2 xi = g.x[i];
    b[2 * i] = g.mass[i] / dt * g.v[i].x;
    b[2 * i + 1] = g.mass[i] / dt * g.v[i].y;
    u[2 * i] = g.v[i].x;
    u[2 * i + 1] = g.v[i].y;
    double vv = g.mass[i] / dt;
    for_faces(g, i, [&](int j, const Edge& e, V2 y) {
      double lrr = lr_ratio(xi - y, e);
      double wv = -0.5 * lrr * (g.mu[i] + g.mu[j]);
      rows[i].push_back(j);
      vals[i].push_back(wv);
      vv -= wv;
    });
    rows[i].push_back(i);
    vals[i].push_back(vv);
  }
  auto apply = [&](const double* in, double* out) {
#pragma omp parallel for
    for (int r = 0; r < 2 * n; ++r) {
      const int i = r / 2, c = r % 2;
      double yr = 0.0;
      for (size_t k = 0; k < rows[i].size(); ++k) yr += vals[i][k] * in[2 * rows[i][k] + c];
      out[r] = yr;
    }
  };
  minres_op(2 * n, apply, b, u, tol, tol, itmax, st);
  for (int i = 0; i < n; ++i) g.v[i] = V2{u[2 * i], u[2 * i + 1]};
  return ST_OK;
}

void find_dv(Grid& g, double dt, double alpha) {  // relaxation.jl:10-25
#pragma omp parallel for
  for (int i = 0; i < g.n; ++i) {
    const V2 xi = g.x[i];
    V2 c = poly_centroid(g.edges[i], xi);
    double rmax = 0.0, rmin = std::numeric_limits<double>::infinity();
    for_faces(g, i, [&](int, const Edge&, V2 y) {
      double r = norm(xi - y);
      rmax = jmax(rmax, r);
      rmin = jmin(rmin, r);
    });
    g.quality[i] = rmin / rmax;
    const M2 D = g.D[i];
    double nD = std::sqrt(D.a11 * D.a11 + D.a21 * D.a21 + D.a12 * D.a12 + D.a22 * D.a22);
    double lambda = alpha * nD / (g.quality[i] * g.quality[i]);
    double s = lambda / (1.0 + dt * lambda);
    g.dv[i] = s * (c - xi);
  }
}

void relaxation_step(Grid& g, double dt, bool rusanov) {  // relaxation.jl:36-73 (without the remesh)
  std::vector<double> newmass(g.n);
#pragma omp parallel for
  for (int i = 0; i < g.n; ++i) {
    const V2 xi = g.x[i];
    const double rp = g.rho[i];
    const V2 vp = g.v[i];
    const double ep = g.e[i];
    double mass = g.mass[i];
    V2 mom = mass * vp;
    double energy = mass * ep;
    for_faces(g, i, [&](int j, const Edge& e, V2 y) {
      if (g.phase[i] != g.phase[j]) return;
      double lrr = lr_ratio(xi - y, e);
      V2 m = midpoint(e);
      V2 z = 0.5 * (xi + y);
      const double rq = g.rho[j];
      const V2 vq = g.v[j];
      const double eq = g.e[j];
      double pdvpq = dot(g.dv[i], xi - y);
      double qdvpq = dot(g.dv[j], xi - y);
      double pdvmz = dot(g.dv[i], m - z);
      double qdvmz = dot(g.dv[j], m - z);
      double k = dt * lrr;
      mass += k * ((pdvmz * rp - qdvmz * rq) - 0.5 * (pdvpq * rp + qdvpq * rq));
      V2 t1 = (pdvmz * rp) * vp - (qdvmz * rq) * vq;
      V2 t2 = (pdvpq * rp) * vp + (qdvpq * rq) * vq;
      mom = mom + k * (t1 - 0.5 * t2);
      energy += k * ((pdvmz * rp * ep - qdvmz * rq * eq) - 0.5 * (pdvpq * rp * ep + qdvpq * rq * eq));
      if (rusanov) {
        double a = jmax(norm(g.dv[i]), norm(g.dv[j]));
        double l = len(e);
        double cr = 0.5 * dt * l * a;
        mass += cr * (rq - rp);
        mom = mom + cr * (rq * vq - rp * vp);
        energy += cr * (rq * eq - rp * ep);
      }
    });
    newmass[i] = mass;
    g.momentum[i] = mom;
    g.energy[i] = energy;
  }
#pragma omp parallel for
  for (int i = 0; i < g.n; ++i) {
    g.mass[i] = newmass[i];
    g.v[i] = V2{g.momentum[i].x / g.mass[i], g.momentum[i].y / g.mass[i]};
    g.e[i] = g.energy[i] / g.mass[i];
    g.x[i] = g.x[i] + dt * g.dv[i];
  }
}

// voronoigrid.jl:181-192
inline double least_positive_residue(double x, double d) { return std::fmod(std::fmod(x, d) + d, d); }
V2 periodic_wrap(const Grid& g, V2 x) {
  double _x = least_positive_residue(x.x - g.bmin.x, g.xperiod) + g.bmin.x;
  double _y = least_positive_residue(x.y - g.bmin.y, g.yperiod) + g.bmin.y;
  V2 r = x;
  if (g.xper) r.x = r.x + (_x - x.x);
  if (g.yper) r.y = r.y + (_y - x.y);
  return r;
}

inline bool isinside_b(const Grid& g, V2 x) {  // geometry.jl:127-129
  return g.bmin.x <= x.x && x.x <= g.bmax.x && g.bmin.y <= x.y && x.y <= g.bmax.y;
}

// move.jl:9-33 (without the remesh).  Returns ST_NAN_VELOCITY on NaN.
int move_particles(Grid& g, double dt) {
  int bad = 0;
#pragma omp parallel for reduction(max : bad)
  for (int i = 0; i < g.n; ++i) {
    auto try_move = [&](int& nanflag) -> bool {
      if (std::isnan(g.v[i].x) || std::isnan(g.v[i].y)) {
        nanflag = 1;
        return true;
      }
      V2 nx = periodic_wrap(g, g.x[i] + dt * g.v[i]);
      if (isinside_b(g, nx)) {
        g.x[i] = nx;
        return true;
      }
      return false;
    };
    int nanflag = 0;
    if (try_move(nanflag)) {
      bad = std::max(bad, nanflag);
      continue;
    }
    for (const auto& e : g.edges[i]) {
      if (e.label >= 0) continue;
      V2 nv = normal_vector(e);
      g.v[i] = g.v[i] - dot(g.v[i], nv) * nv;
    }
    if (try_move(nanflag)) {
      bad = std::max(bad, nanflag);
      continue;
    }
    g.v[i] = V2{0.0, 0.0};
    try_move(nanflag);
    bad = std::max(bad, nanflag);
  }
  return bad ? ST_NAN_VELOCITY : ST_OK;
}

// ----------------------------------------------------- multiphase projector
// relaxation.jl:91-123 operator applied to xin.
void mp_mul(const Grid& g, const double* xin, double* res, std::vector<V2>& tmp) {
#pragma omp parallel for
  for (int i = 0; i < g.n; ++i) {
    V2 t{0.0, 0.0};
    const V2 xi = g.x[i];
    for_faces(g, i, [&](int j, const Edge& e, V2 y) {
      if (g.phase[i] == g.phase[j]) return;
      double lrr = lr_ratio(xi - y, e);
      V2 m = midpoint(e);
      t = t - (lrr * (xin[i] - xin[j])) * (m - xi);
    });
    double A = poly_area(g.edges[i], xi);
    tmp[i] = V2{t.x / A, t.y / A};
  }
#pragma omp parallel for
  for (int i = 0; i < g.n; ++i) {
    double r = 0.0;
    const V2 xi = g.x[i];
    for_faces(g, i, [&](int j, const Edge& e, V2 y) {
      if (g.phase[i] == g.phase[j]) return;
      double lrr = lr_ratio(xi - y, e);
      V2 m = midpoint(e);
      V2 z = 0.5 * (xi + y);
      r -= lrr * (dot(tmp[i] - tmp[j], m - z) - 0.5 * dot(tmp[i] + tmp[j], xi - y));
    });
    res[i] = r;
  }
}

}  // namespace

// =================================================================== C ABI

extern "C" {

struct lvref_grid_params {
  double xmin[2], xmax[2];
  double dr, h, r_max;
  int32_t xperiodic, yperiodic;
  int32_t max_edges;
};

enum {
  F_X = 0, F_V = 1, F_E = 2, F_P = 3, F_RHO = 4, F_C2 = 5, F_DV = 6, F_MASS = 7, F_MOMENTUM = 8,
  F_ENERGY = 9, F_PHASE = 10, F_QUALITY = 11, F_D = 12, F_MU = 13, F_T = 14, F_K = 15, F_CV = 16
};

void* lvref_create(const lvref_grid_params* p, int n) {
  Grid* g = new Grid();
  g->bmin = V2{p->xmin[0], p->xmin[1]};
  g->bmax = V2{p->xmax[0], p->xmax[1]};
  g->dr = p->dr;
  g->h = p->h;
  g->r_max = p->r_max;
  g->xper = p->xperiodic != 0;
  g->yper = p->yperiodic != 0;
  g->max_edges = p->max_edges > 0 ? p->max_edges : 64;
  double rx = g->xper ? g->r_max : 0.0, ry = g->yper ? g->r_max : 0.0;
  g->cmin = V2{g->bmin.x - rx, g->bmin.y - ry};
  g->cmax = V2{g->bmax.x + rx, g->bmax.y + ry};
  g->xperiod = g->bmax.x - g->bmin.x;
  g->yperiod = g->bmax.y - g->bmin.y;
  g->rr_max = g->r_max * g->r_max;
  g->origin = g->cmin - V2{g->h, g->h};
  g->n1 = (int64_t)std::floor((g->cmax.x - g->cmin.x) / g->h) + 3;
  g->n2 = (int64_t)std::floor((g->cmax.y - g->cmin.y) / g->h) + 3;
  g->cells.assign((size_t)(g->n1 * g->n2), {});
  build_path(*g);
  g->n = n;
  g->x.assign(n, V2{0, 0});
  g->v.assign(n, V2{0, 0});
  g->dv.assign(n, V2{0, 0});
  g->momentum.assign(n, V2{0, 0});
  for (auto* f : {&g->rho, &g->e, &g->P, &g->c2, &g->mass, &g->energy, &g->quality, &g->mu, &g->T, &g->kc, &g->cV})
    f->assign(n, 0.0);
  g->phase.assign(n, 0);
  g->D.assign(n, M2{0, 0, 0, 0});
  g->edges.assign(n, {});
  return g;
}

void lvref_destroy(void* h) { delete static_cast<Grid*>(h); }

int lvref_num_threads(int nt) {
#ifdef _OPENMP
  if (nt > 0) omp_set_num_threads(nt);
  return omp_get_max_threads();
#else
  (void)nt;
  return 1;
#endif
}

int lvref_cell_dims(void* h, int64_t* n1, int64_t* n2) {
  Grid* g = static_cast<Grid*>(h);
  *n1 = g->n1;
  *n2 = g->n2;
  return 0;
}

// Copies out the visited prefix of the cell path: offsets (i1,i2) and rr.
int lvref_path(void* h, int64_t* i1, int64_t* i2, double* rr, int cap) {
  Grid* g = static_cast<Grid*>(h);
  int n = (int)g->path.size();
  for (int k = 0; k < n && k < cap; ++k) {
    i1[k] = g->path[k].i1;
    i2[k] = g->path[k].i2;
    rr[k] = g->path[k].rr;
  }
  return n;
}

int lvref_set_field(void* h, int f, const double* src) {
  Grid* g = static_cast<Grid*>(h);
  const int n = g->n;
  switch (f) {
    case F_X: for (int i = 0; i < n; ++i) g->x[i] = V2{src[2 * i], src[2 * i + 1]}; break;
    case F_V: for (int i = 0; i < n; ++i) g->v[i] = V2{src[2 * i], src[2 * i + 1]}; break;
    case F_DV: for (int i = 0; i < n; ++i) g->dv[i] = V2{src[2 * i], src[2 * i + 1]}; break;
    case F_MOMENTUM: for (int i = 0; i < n; ++i) g->momentum[i] = V2{src[2 * i], src[2 * i + 1]}; break;
    case F_D: for (int i = 0; i < n; ++i) g->D[i] = M2{src[4 * i], src[4 * i + 1], src[4 * i + 2], src[4 * i + 3]}; break;
    case F_PHASE: for (int i = 0; i < n; ++i) g->phase[i] = (int32_t)src[i]; break;
    case F_E: std::memcpy(g->e.data(), src, 8 * n); break;
    case F_P: std::memcpy(g->P.data(), src, 8 * n); break;
    case F_RHO: std::memcpy(g->rho.data(), src, 8 * n); break;
    case F_C2: std::memcpy(g->c2.data(), src, 8 * n); break;
    case F_MASS: std::memcpy(g->mass.data(), src, 8 * n); break;
    case F_ENERGY: std::memcpy(g->energy.data(), src, 8 * n); break;
    case F_QUALITY: std::memcpy(g->quality.data(), src, 8 * n); break;
    case F_MU: std::memcpy(g->mu.data(), src, 8 * n); break;
    case F_T: std::memcpy(g->T.data(), src, 8 * n); break;
    case F_K: std::memcpy(g->kc.data(), src, 8 * n); break;
    case F_CV: std::memcpy(g->cV.data(), src, 8 * n); break;
    default: return ST_BAD_ARGUMENT;
  }
  return 0;
}

int lvref_get_field(void* h, int f, double* dst) {
  Grid* g = static_cast<Grid*>(h);
  const int n = g->n;
  switch (f) {
    case F_X: for (int i = 0; i < n; ++i) { dst[2 * i] = g->x[i].x; dst[2 * i + 1] = g->x[i].y; } break;
    case F_V: for (int i = 0; i < n; ++i) { dst[2 * i] = g->v[i].x; dst[2 * i + 1] = g->v[i].y; } break;
    case F_DV: for (int i = 0; i < n; ++i) { dst[2 * i] = g->dv[i].x; dst[2 * i + 1] = g->dv[i].y; } break;
    case F_MOMENTUM: for (int i = 0; i < n; ++i) { dst[2 * i] = g->momentum[i].x; dst[2 * i + 1] = g->momentum[i].y; } break;
    case F_D: for (int i = 0; i < n; ++i) { dst[4 * i] = g->D[i].a11; dst[4 * i + 1] = g->D[i].a21; dst[4 * i + 2] = g->D[i].a12; dst[4 * i + 3] = g->D[i].a22; } break;
    case F_PHASE: for (int i = 0; i < n; ++i) dst[i] = g->phase[i]; break;
    case F_E: std::memcpy(dst, g->e.data(), 8 * n); break;
    case F_P: std::memcpy(dst, g->P.data(), 8 * n); break;
    case F_RHO: std::memcpy(dst, g->rho.data(), 8 * n); break;
    case F_C2: std::memcpy(dst, g->c2.data(), 8 * n); break;
    case F_MASS: std::memcpy(dst, g->mass.data(), 8 * n); break;
    case F_ENERGY: std::memcpy(dst, g->energy.data(), 8 * n); break;
    case F_QUALITY: std::memcpy(dst, g->quality.data(), 8 * n); break;
    case F_MU: std::memcpy(dst, g->mu.data(), 8 * n); break;
    case F_T: std::memcpy(dst, g->T.data(), 8 * n); break;
    case F_K: std::memcpy(dst, g->kc.data(), 8 * n); break;
    case F_CV: std::memcpy(dst, g->cV.data(), 8 * n); break;
    default: return ST_BAD_ARGUMENT;
  }
  return 0;
}

int lvref_remesh(void* h) { return remesh(*static_cast<Grid*>(h)); }

// Cell-list contents: starts[n1*n2+1] (CSR) and items (particle indices in
// insertion order); returns the item count (or the needed size if cap is short).
int64_t lvref_cell_items(void* h, int64_t* starts, int32_t* items, int64_t cap) {
  Grid* g = static_cast<Grid*>(h);
  int64_t total = 0;
  for (size_t c = 0; c < g->cells.size(); ++c) {
    if (starts) starts[c] = total;
    for (int32_t v : g->cells[c]) {
      if (items && total < cap) items[total] = v;
      ++total;
    }
  }
  if (starts) starts[g->cells.size()] = total;
  return total;
}

// Geometry after remesh: per polygon the edge count, edges (v1x v1y v2x v2y)
// in the stored order, labels, area and centroid.  Arrays are [n][maxe].
int lvref_get_edges(void* h, int maxe, int32_t* counts, double* verts, int32_t* labels, double* area,
                    double* centroid) {
  Grid* g = static_cast<Grid*>(h);
  int worst = 0;
  for (int i = 0; i < g->n; ++i) {
    const auto& E = g->edges[i];
    counts[i] = (int32_t)E.size();
    if ((int)E.size() > maxe) {
      worst = ST_EDGE_OVERFLOW;
      continue;
    }
    for (size_t k = 0; k < E.size(); ++k) {
      double* vv = verts + ((size_t)i * maxe + k) * 4;
      vv[0] = E[k].v1.x;
      vv[1] = E[k].v1.y;
      vv[2] = E[k].v2.x;
      vv[3] = E[k].v2.y;
      labels[(size_t)i * maxe + k] = (int32_t)E[k].label;
    }
    if (area) area[i] = poly_area(E, g->x[i]);
    if (centroid) {
      V2 c = poly_centroid(E, g->x[i]);
      centroid[2 * i] = c.x;
      centroid[2 * i + 1] = c.y;
    }
  }
  return worst;
}

// Per-face quantities in the iteration order of `neighbors` (iterators.jl:23-33):
// rowptr[n+1], nbr, lrr = lr_ratio(x - y, e), mid = midpoint(e), y.
int64_t lvref_get_faces(void* h, int64_t* rowptr, int32_t* nbr, double* lrr, double* mid, double* ypos,
                        double* elen, int64_t cap) {
  Grid* g = static_cast<Grid*>(h);
  int64_t k = 0;
  for (int i = 0; i < g->n; ++i) {
    if (rowptr) rowptr[i] = k;
    const V2 xi = g->x[i];
    for_faces(*g, i, [&](int j, const Edge& e, V2 y) {
      if (nbr && k < cap) {
        nbr[k] = j;
        lrr[k] = lr_ratio(xi - y, e);
        V2 m = midpoint(e);
        mid[2 * k] = m.x;
        mid[2 * k + 1] = m.y;
        ypos[2 * k] = y.x;
        ypos[2 * k + 1] = y.y;
        if (elen) elen[k] = len(e);
      }
      ++k;
    });
  }
  if (rowptr) rowptr[g->n] = k;
  return k;
}

// Half-plane clip of a single polygon (known-answer tests): edges in/out as
// [k][4] plus labels; returns the new edge count (or -1 on overflow) and the
// cut flag through *cut.
int lvref_clip_polygon(const double* px, const double* y, int64_t label, int nedges, double* verts, int32_t* labels,
                       int cap, int* cut) {
  std::vector<Edge> E;
  for (int k = 0; k < nedges; ++k)
    E.push_back(Edge{V2{verts[4 * k], verts[4 * k + 1]}, V2{verts[4 * k + 2], verts[4 * k + 3]}, labels[k]});
  int r = voronoicut_poly(E, V2{px[0], px[1]}, V2{y[0], y[1]}, label, cap);
  if (r < 0) return -1;
  *cut = r;
  for (size_t k = 0; k < E.size(); ++k) {
    verts[4 * k] = E[k].v1.x;
    verts[4 * k + 1] = E[k].v1.y;
    verts[4 * k + 2] = E[k].v2.x;
    verts[4 * k + 3] = E[k].v2.y;
    labels[k] = (int32_t)E[k].label;
  }
  return (int)E.size();
}

int lvref_ideal_eos(void* h, double gamma, double Pmin) { ideal_eos(*static_cast<Grid*>(h), gamma, Pmin); return 0; }
int lvref_stiffened_eos(void* h, double gamma, double P0) { stiffened_eos(*static_cast<Grid*>(h), gamma, P0); return 0; }
int lvref_find_rho(void* h) { find_rho(*static_cast<Grid*>(h)); return 0; }
int lvref_gravity_step(void* h, double gx, double gy, double dt) { gravity_step(*static_cast<Grid*>(h), V2{gx, gy}, dt); return 0; }
int lvref_pressure_step(void* h, double dt) { pressure_step(*static_cast<Grid*>(h), dt); return 0; }
int lvref_find_D(void* h) { find_D(*static_cast<Grid*>(h)); return 0; }
int lvref_viscous_step(void* h, double dt, int av) { viscous_step(*static_cast<Grid*>(h), dt, av != 0); return 0; }
int lvref_bdary_friction(void* h, const double* vwall, double dt) { bdary_friction(*static_cast<Grid*>(h), vwall, dt); return 0; }

int lvref_ideal_temperature(void* h) { ideal_temperature(*static_cast<Grid*>(h)); return 0; }
int lvref_fourier_step(void* h, double dt) { fourier_step(*static_cast<Grid*>(h), dt); return 0; }
int lvref_heat_from_bdary(void* h, double dt, const double* Tb) { return heat_from_bdary(*static_cast<Grid*>(h), dt, Tb); }
int lvref_viscous_solve(void* h, double dt, double tol, int itmax, SolveStats* st) {
  return viscous_solve(*static_cast<Grid*>(h), dt, tol, itmax, st);
}

// The boundary edges in the per-edge order: midpoints mid[nb][2] =
// midpoint(e) and labels; returns nb (arrays filled when cap >= nb).
int64_t lvref_boundary_edges(void* h, double* mid, int32_t* lab, int64_t cap) {
  Grid* g = static_cast<Grid*>(h);
  int64_t q = 0;
  for (int i = 0; i < g->n; ++i)
    for (const auto& e : g->edges[i]) {
      if (e.label >= 0) continue;
      if (q < cap) {
        const V2 m = 0.5 * (e.v1 + e.v2);
        if (mid) {
          mid[2 * q] = m.x;
          mid[2 * q + 1] = m.y;
        }
        if (lab) lab[q] = (int32_t)e.label;
      }
      ++q;
    }
  return q;
}

// Per-edge boundary values for refresh_rhs and bdary_friction (vb NULL: back
// to the label table); act may be NULL (every edge).
int lvref_set_edge_values(void* h, int64_t nb, const double* vb, const uint8_t* act) {
  Grid* g = static_cast<Grid*>(h);
  g->edge_mode = vb != nullptr;
  g->edge_vel.assign(vb ? nb : 0, V2{0.0, 0.0});
  for (int64_t q = 0; vb && q < nb; ++q) g->edge_vel[q] = V2{vb[2 * q], vb[2 * q + 1]};
  g->edge_act.assign(act ? act : nullptr, act ? act + nb : nullptr);
  return 0;
}
int lvref_find_dv(void* h, double dt, double alpha) { find_dv(*static_cast<Grid*>(h), dt, alpha); return 0; }

int lvref_relaxation_step(void* h, double dt, int rusanov) {
  Grid* g = static_cast<Grid*>(h);
  relaxation_step(*g, dt, rusanov != 0);
  return remesh(*g);
}
int lvref_relax_no_remesh(void* h, double dt, int rusanov) {
  relaxation_step(*static_cast<Grid*>(h), dt, rusanov != 0);
  return 0;
}

int lvref_move(void* h, double dt) {
  Grid* g = static_cast<Grid*>(h);
  int st = move_particles(*g, dt);
  if (st) return st;
  return remesh(*g);
}
int lvref_move_no_remesh(void* h, double dt) { return move_particles(*static_cast<Grid*>(h), dt); }

// Pressure operator (pressure.jl:104-117): diag[n], rowptr[n+1], col, w.
int64_t lvref_pressure_operator(void* h, double dt, double* diag, int64_t* rowptr, int32_t* col, double* w,
                                int64_t cap) {
  Grid* g = static_cast<Grid*>(h);
  refresh_operator(*g, dt);
  int64_t k = 0;
  for (int i = 0; i < g->n; ++i) {
    if (diag) diag[i] = g->diag[i];
    if (rowptr) rowptr[i] = k;
    for (size_t t = 0; t < g->op_nbr[i].size(); ++t, ++k)
      if (col && k < cap) {
        col[k] = g->op_nbr[i][t];
        w[k] = g->op_w[i][t];
      }
  }
  if (rowptr) rowptr[g->n] = k;
  return k;
}

// RHS refresh (pressure.jl:162-203) with the operator already refreshed.
int lvref_pressure_rhs(void* h, double dt, int gp_step, const double* vbc, double* b, double* gp) {
  Grid* g = static_cast<Grid*>(h);
  refresh_rhs(*g, dt, gp_step != 0, vbc);
  for (int i = 0; i < g->n; ++i) {
    if (b) b[i] = g->b[i];
    if (gp) {
      gp[2 * i] = g->GP[i].x;
      gp[2 * i + 1] = g->GP[i].y;
    }
  }
  return 0;
}

// Operator application y = A x with the operator last refreshed.
int lvref_operator_apply(void* h, const double* xin, double* y) {
  op_mul(*static_cast<Grid*>(h), xin, y);
  return 0;
}

// The GPU solver's initial guess of a sweep (not part of the reference,
// whose MINRES starts from the previous sweep's P): the start x moves to
// x + c1 d1 + c2 D, the Galerkin projection of the error onto span{d1, D} in
// the A-norm, d1 = x - prev (the last sweep's change, sweeps >= 2), D = the
// change of this sweep in the previous call (if it ran this sweep).  res =
// b - A x is evaluated on sweep 1 and taken as b - bprev on the others (the
// previous solve's residual, below its tolerance, is dropped); projected to
// zero mean when the operator is singular.  A nearly dependent pair (det <=
// 1e-6 a11 a22) keeps the single direction that lowers the error more;
// coefficients outside (-4, 4) or undefined give the plain warm start.
// prev and bprev receive x and b before the move.
void sweep_guess(const Grid& g, std::vector<double>& x, std::vector<double>& prev, std::vector<double>& bprev,
                 const std::vector<double>* D, int it) {
  const int n = g.n;
  const bool has1 = it >= 2, has2 = D != nullptr;
  std::vector<double> res(n), d1(n, 0.0);
  if (has1) {
    for (int i = 0; i < n; ++i) {
      d1[i] = x[i] - prev[i];
      res[i] = g.b[i] - bprev[i];
    }
  } else {
    std::vector<double> Ax(n);
    op_mul(g, x.data(), Ax.data());
    for (int i = 0; i < n; ++i) res[i] = g.b[i] - Ax[i];
  }
  prev = x;
  bprev = g.b;
  if (!has1 && !has2) return;
  bool singular = true;
  for (int i = 0; i < n; ++i)
    if (g.diag[i] != 0.0) {
      singular = false;
      break;
    }
  if (singular && n > 0) {
    double sr = 0.0;
    for (int i = 0; i < n; ++i) sr += res[i];
    for (int i = 0; i < n; ++i) res[i] -= sr / n;
  }
  std::vector<double> A1(n, 0.0), A2(n, 0.0);
  double r1 = 0.0, r2 = 0.0, a11 = 0.0, a12 = 0.0, a22 = 0.0;
  if (has1) {
    op_mul(g, d1.data(), A1.data());
    r1 = bdot(res.data(), d1.data(), n);
    a11 = bdot(d1.data(), A1.data(), n);
  }
  if (has2) {
    op_mul(g, D->data(), A2.data());
    r2 = bdot(res.data(), D->data(), n);
    a22 = bdot(D->data(), A2.data(), n);
    if (has1) a12 = bdot(d1.data(), A2.data(), n);
  }
  double c1 = 0.0, c2 = 0.0;
  const bool u1 = has1 && a11 > 0.0, u2 = has2 && a22 > 0.0;
  const double det = a11 * a22 - a12 * a12;
  if (u1 && u2 && det > 1e-6 * a11 * a22) {
    c1 = (r1 * a22 - r2 * a12) / det;
    c2 = (a11 * r2 - a12 * r1) / det;
  } else if (u1 && (!u2 || r1 * r1 / a11 >= r2 * r2 / a22)) {
    c1 = r1 / a11;
  } else if (u2) {
    c2 = r2 / a22;
  }
  if (!(c1 > -4.0 && c1 < 4.0 && c2 > -4.0 && c2 < 4.0)) c1 = c2 = 0.0;
  for (int i = 0; i < n; ++i) x[i] += c1 * d1[i] + (has2 ? c2 * (*D)[i] : 0.0);
}

// find_pressure! (pressure.jl:215-224).  method 0: MINRES (atol = rtol = tol),
// method 1: Jacobi-PCG with ||r|| <= tol*||b||, method 2: the same PCG from
// the GPU solver's Galerkin initial guess (sweep_guess).  stats[niter]
// receives one record per fixed-point sweep.
int lvref_find_pressure(void* h, double dt, int niter, const double* vbc, int method, double tol, int itmax,
                        SolveStats* stats) {
  Grid* g = static_cast<Grid*>(h);
  refresh_operator(*g, dt);
  std::vector<double> prev, bprev;
  if ((int)g->sweep_n != g->n) g->sweep_inc.clear();
  for (int it = 1; it <= niter; ++it) {
    refresh_rhs(*g, dt, it > 1, vbc);
    std::vector<double> x = g->Psol;
    if (method == 2) sweep_guess(*g, x, prev, bprev, it <= (int)g->sweep_inc.size() ? &g->sweep_inc[it - 1] : nullptr, it);
    SolveStats st{};
    if (method == 0)
      minres_solve(*g, g->b, x, tol, tol, itmax, &st);
    else
      pcg_solve(*g, g->b, x, tol, itmax, &st);
    if (stats) stats[it - 1] = st;
    if (method == 2) {
      // this sweep's change, for the same sweep of the next call
      std::vector<double> dd(g->n);
      for (int i = 0; i < g->n; ++i) dd[i] = (double)(float)(x[i] - g->P[i]);
      if ((int)g->sweep_inc.size() < it) g->sweep_inc.resize(it);
      g->sweep_inc[it - 1] = dd;
      g->sweep_n = g->n;
    }
    for (int i = 0; i < g->n; ++i) g->P[i] = x[i];
  }
  return 0;
}

// One linear solve on the current operator: method as above.
int lvref_solve(void* h, const double* b, double* x, int method, double tol, int itmax, SolveStats* st) {
  Grid* g = static_cast<Grid*>(h);
  std::vector<double> bv(b, b + g->n), xv(x, x + g->n);
  if (method == 0)
    minres_solve(*g, bv, xv, tol, tol, itmax, st);
  else
    pcg_solve(*g, bv, xv, tol, itmax, st);
  std::memcpy(x, xv.data(), 8 * g->n);
  return 0;
}

// multiphase_projection! (relaxation.jl:155-206); MINRES atol = rtol = 1e-4, itmax 200.
int lvref_multiphase_projection(void* h, double quality_threshold, double tol, int itmax, SolveStats* st) {
  Grid* g = static_cast<Grid*>(h);
  const int n = g->n;
  std::vector<double> b(n, 0.0), q(n, 0.0);
#pragma omp parallel for
  for (int i = 0; i < n; ++i) {
    double bi = 0.0;
    const V2 xi = g->x[i];
    for_faces(*g, i, [&](int j, const Edge& e, V2 y) {
      if (g->phase[i] == g->phase[j]) return;
      double lrr = lr_ratio(xi - y, e);
      V2 m = midpoint(e);
      V2 z = 0.5 * (xi + y);
      bi -= lrr * (dot(g->dv[i] - g->dv[j], m - z) - 0.5 * dot(g->dv[i] + g->dv[j], xi - y));
    });
    b[i] = bi;
  }
  // MINRES on the projector: reuse minres_solve through a temporary operator
  // view is not possible (it applies the pressure operator), so run it inline.
  std::vector<V2> tmp(n);
  std::vector<double> r1(n), r2(n), y(n), v(n), w(n, 0.0), w1(n), w2(n, 0.0);
  r1 = b;
  y = r1;
  double beta1 = std::sqrt(bdot(r1.data(), y.data(), n));
  int itn = 0;
  bool solved = beta1 == 0.0;
  if (!solved) {
    r2 = r1;
    double oldb = 0.0, beta = beta1, dbar = 0.0, epsln = 0.0, phibar = beta1, cs = -1.0, sn = 0.0, tnorm2 = 0.0;
    const double eps = std::numeric_limits<double>::epsilon();
    double tl = tol + tol * beta1;
    while (itn < itmax) {
      ++itn;
      double s = 1.0 / beta;
      for (int i = 0; i < n; ++i) v[i] = s * y[i];
      mp_mul(*g, v.data(), y.data(), tmp);
      if (itn >= 2)
        for (int i = 0; i < n; ++i) y[i] -= (beta / oldb) * r1[i];
      double alfa = bdot(v.data(), y.data(), n);
      for (int i = 0; i < n; ++i) y[i] -= (alfa / beta) * r2[i];
      r1.swap(r2);
      r2 = y;
      oldb = beta;
      beta = std::sqrt(std::max(0.0, bdot(r2.data(), y.data(), n)));
      tnorm2 += alfa * alfa + oldb * oldb + beta * beta;
      double oldeps = epsln, delta = cs * dbar + sn * alfa, gbar = sn * dbar - cs * alfa;
      epsln = sn * beta;
      dbar = -cs * beta;
      double root = std::sqrt(gbar * gbar + dbar * dbar);
      double gamma = std::max(std::sqrt(gbar * gbar + beta * beta), eps);
      cs = gbar / gamma;
      sn = beta / gamma;
      double phi = cs * phibar;
      phibar = sn * phibar;
      double denom = 1.0 / gamma;
      w1.swap(w2);
      w2.swap(w);
      for (int i = 0; i < n; ++i) {
        w[i] = (v[i] - oldeps * w1[i] - delta * w2[i]) * denom;
        q[i] += phi * w[i];
      }
      double Anorm = std::sqrt(tnorm2), Arnorm = phibar * root;
      if (phibar <= tl || beta == 0.0 || (Anorm > 0 && phibar > 0 && Arnorm / (Anorm * phibar) <= tol)) {
        solved = true;
        break;
      }
    }
  }
  if (st) {
    st->iterations = itn;
    st->converged = solved ? 1 : 0;
    st->rel_residual = 0.0;
  }
  std::vector<V2> ndv(g->dv);
#pragma omp parallel for
  for (int i = 0; i < n; ++i) {
    if (g->quality[i] < quality_threshold) continue;
    const V2 xi = g->x[i];
    V2 d = g->dv[i];
    double A = poly_area(g->edges[i], xi);
    for_faces(*g, i, [&](int j, const Edge& e, V2 y) {
      if (g->phase[i] == g->phase[j]) return;
      V2 m = midpoint(e);
      double c = lr_ratio(xi - y, e) * (q[i] - q[j]);
      V2 t = c * (m - xi);
      d = d + V2{t.x / A, t.y / A};
    });
    ndv[i] = d;
  }
  g->dv = ndv;
  return 0;
}

// ------------------------------------------------------------ moving least squares

// The reference's cell path in full: every offset of the (2 n - 1)^2 range
// (neighborlist.jl:29-41, swapped n1/n2 bounds), ordered as build_path
// orders its prefix, cut after the first node with rr > bound.
static std::vector<PathNode> path_upto(const Grid& g, double bound) {
  std::vector<PathNode> all;
  for (int64_t i2 = 1 - g.n1; i2 <= g.n1 - 1; ++i2)
    for (int64_t i1 = 1 - g.n2; i1 <= g.n2 - 1; ++i1) {
      int64_t a = std::max<int64_t>(0, std::llabs(i1) - 1), c = std::max<int64_t>(0, std::llabs(i2) - 1);
      double rr = (g.h * g.h) * (double)(a * a + c * c);
      all.push_back({i1, i2, i1 * i1 + i2 * i2, rr});
    }
  std::stable_sort(all.begin(), all.end(), [](const PathNode& p, const PathNode& q) { return p.keysq < q.keysq; });
  std::stable_sort(all.begin(), all.end(), [](const PathNode& p, const PathNode& q) { return p.rr < q.rr; });
  std::vector<PathNode> out;
  for (const auto& nd : all) {
    out.push_back(nd);
    if (nd.rr > bound) break;
  }
  return out;
}

// voronoigrid.jl:154-178; -1 when no polygon is met
static int nearest_polygon(const Grid& g, const std::vector<PathNode>& path, V2 x) {
  int64_t k1, k2;
  if (!findkey(g, x, k1, k2)) return -1;
  double rr_best = INFINITY;
  int i_best = -1;
  for (const auto& nd : path) {
    if (nd.rr > rr_best) break;
    const int64_t c1 = k1 + nd.i1, c2 = k2 + nd.i2;
    if (c1 < 1 || c1 > g.n1 || c2 < 1 || c2 > g.n2) continue;
    for (int32_t i : g.cells[(c1 - 1) + g.n1 * (c2 - 1)]) {
      const double prr = norm_squared(g.x[i] - x);
      if (prr < rr_best) {
        rr_best = prr;
        i_best = i;
      }
    }
  }
  return i_best;
}

// power_vector (movingls.jl:26-36) for 2, 5 or 9 coefficients
static int power_vector(int nc, V2 d, double* pv) {
  pv[0] = d.x;
  pv[1] = d.y;
  if (nc >= 5) {
    pv[2] = d.x * d.x;
    pv[3] = d.x * d.y;
    pv[4] = d.y * d.y;
  }
  if (nc >= 9) {
    pv[5] = (d.x * d.x) * d.x;
    pv[6] = (d.x * d.x) * d.y;
    pv[7] = (d.x * d.y) * d.y;
    pv[8] = (d.y * d.y) * d.y;
  }
  return nc;
}

// R \ a: the explicit 2x2 formula, Gaussian elimination with partial
// pivoting otherwise
static void small_solve(int nc, double* R, double* a) {
  if (nc == 2) {
    const double d = R[0] * R[3] - R[2] * R[1];  // R column-major: R[k + nc*l]
    const double b0 = a[0], b1 = a[1];
    a[0] = (R[3] * b0 - R[2] * b1) / d;
    a[1] = (R[0] * b1 - R[1] * b0) / d;
    return;
  }
  for (int k = 0; k < nc; ++k) {
    int piv = k;
    for (int r = k + 1; r < nc; ++r)
      if (std::fabs(R[r + nc * k]) > std::fabs(R[piv + nc * k])) piv = r;
    if (piv != k) {
      for (int c = 0; c < nc; ++c) std::swap(R[k + nc * c], R[piv + nc * c]);
      std::swap(a[k], a[piv]);
    }
    for (int r = k + 1; r < nc; ++r) {
      const double f = R[r + nc * k] / R[k + nc * k];
      for (int c = k; c < nc; ++c) R[r + nc * c] -= f * R[k + nc * c];
      a[r] -= f * a[k];
    }
  }
  for (int k = nc - 1; k >= 0; --k) {
    double t = a[k];
    for (int c = k + 1; c < nc; ++c) t -= R[k + nc * c] * a[c];
    a[k] = t / R[k + nc * k];
  }
}

// movingls (movingls.jl:52-86) with gaussian_kernel (:22-24), for polygon i
// and the per-polygon values f
static void movingls(const Grid& g, const std::vector<PathNode>& path, int nc, int i, const double* f, double h,
                     double* out) {
  double a[9] = {0}, R[81] = {0}, pv[9];
  const V2 px = g.x[i];
  const double fp = f[i];
  int64_t k1, k2;
  if (findkey(g, px, k1, k2)) {
    for (const auto& nd : path) {
      if (nd.rr > h) break;
      const int64_t c1 = k1 + nd.i1, c2 = k2 + nd.i2;
      if (c1 < 1 || c1 > g.n1 || c2 < 1 || c2 > g.n2) continue;
      for (int32_t j : g.cells[(c1 - 1) + g.n1 * (c2 - 1)]) {
        const V2 y = px + get_arrow(g, g.x[j], px);
        if (veq(px, y)) continue;
        const double r = norm(px - y);
        if (r < h) {
          const double q = r / h;
          const double ker = std::exp(-0.5 * (q * q)) / std::sqrt((2.0 * M_PI) * (h * h));
          power_vector(nc, y - px, pv);
          const double s = ker * (f[j] - fp);
          for (int k = 0; k < nc; ++k) a[k] += s * pv[k];
          for (int l = 0; l < nc; ++l)
            for (int k = 0; k < nc; ++k) R[k + nc * l] += (ker * pv[k]) * pv[l];
        }
      }
    }
  }
  small_solve(nc, R, a);
  for (int k = 0; k < nc; ++k) out[k] = a[k];
}

int lvref_nearest_polygon(void* hdl, int m, const double* pts, int32_t* out) {
  const Grid& g = *static_cast<Grid*>(hdl);
  const auto path = path_upto(g, INFINITY);
  for (int q = 0; q < m; ++q) out[q] = nearest_polygon(g, path, V2{pts[2 * q], pts[2 * q + 1]});
  return 0;
}

// order 1, 2, 3: linear, quadratic, cubic; polys NULL: every polygon
int lvref_movingls(void* hdl, int order, int m, const int32_t* polys, const double* f, double h, double* coeffs) {
  const Grid& g = *static_cast<Grid*>(hdl);
  const int nc = order == 1 ? 2 : (order == 2 ? 5 : 9);
  const auto path = path_upto(g, h);
  for (int q = 0; q < m; ++q) movingls(g, path, nc, polys ? polys[q] : q, f, h, coeffs + (size_t)nc * q);
  return 0;
}

// point_value (movingls.jl:140-146): nearest polygon, linear expansion with h = grid.h
int lvref_point_value(void* hdl, int m, const double* pts, const double* f, double* out) {
  const Grid& g = *static_cast<Grid*>(hdl);
  const auto pnear = path_upto(g, INFINITY);
  const auto pls = path_upto(g, g.h);
  for (int q = 0; q < m; ++q) {
    const V2 x{pts[2 * q], pts[2 * q + 1]};
    const int i = nearest_polygon(g, pnear, x);
    if (i < 0) {
      out[q] = NAN;
      continue;
    }
    double L[2];
    movingls(g, pls, 2, i, f, g.h, L);
    const V2 d = x - g.x[i];
    out[q] = f[i] + (L[0] * d.x + L[1] * d.y);
  }
  return 0;
}

}  // extern "C"
