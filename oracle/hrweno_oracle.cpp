// hrweno_oracle.cpp - CPU restatement of HR-WENO's hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity oracle for the GB300 kernels: only the
// tests, the smoke check and the CPU-baseline leg of the benchmark load it.  The product
// library never links or calls it.
//
// It restates, in the reference's own operation order, the Fortran library
// HugoMVale/HR-WENO (no Fortran compiler exists in the build container, so the reference
// itself cannot be built here).  Every function cites the reference file:line it follows.
// It is templated on the real type so that the same code gives the REAL32 / REAL64 /
// REAL128 builds of the reference (src/hrweno_kinds.F90:9-17); REAL128 is the
// high-precision yardstick.  Build with -ffp-contract=off so that no multiply-add is fused
// (the reference's x86-64 gfortran build uses SSE2 and fuses none).
//
// The parity of this restatement is pinned by the reference's own known-answer tests,
// ported to tests/test_oracle_kat.py (test/test_hrweno.f90, test/test_fluxes.f90,
// test/test_tvdode.f90).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../include/hrweno_gpu.h"

#ifdef _OPENMP
#include <omp.h>
// The reference's cell loop is `do concurrent` (src/hrweno_weno.f90:174) and every stage
// combine is an elementwise array expression, so splitting these loops over threads leaves
// each element's arithmetic, and therefore every result bit, unchanged.
#define ORC_PARFOR _Pragma("omp parallel for schedule(static)")
#else
#define ORC_PARFOR
#endif

#if defined(__x86_64__) || defined(__i386__)
typedef __float128 qreal;
#else
typedef long double qreal;  // IEEE binary128 on aarch64
#endif

namespace orc {

static thread_local std::string g_msg;

// ---------------------------------------------------------------------------------------
// Tables d1/d2/d3 and c1/c2/c3 (src/hrweno_weno.f90:11-21).  c(j, r) with j = 0..k-1 and
// r = -1..k-1 is stored at [j + k*(r+1)]: the Fortran column-major reshape order.
// ---------------------------------------------------------------------------------------
template <class T>
static void tables(int k, T* d, T* c) {
  if (k == 1) {
    d[0] = T(1);
    c[0] = T(1); c[1] = T(1);
  } else if (k == 2) {
    d[0] = T(2) / 3; d[1] = T(1) / 3;
    const T cc[6] = {T(3) / 2, T(-1) / 2, T(1) / 2, T(1) / 2, T(-1) / 2, T(3) / 2};
    for (int q = 0; q < 6; ++q) c[q] = cc[q];
  } else {
    d[0] = T(3) / 10; d[1] = T(6) / 10; d[2] = T(1) / 10;
    // Fortran literals 0.3_rk, 0.6_rk, 0.1_rk are the nearest values of the decimal
    // constants, which is what T(3)/10 etc. give for a correctly rounded division.
    const T cc[12] = {T(11) / 6, T(-7) / 6, T(1) / 3,  T(1) / 3,  T(5) / 6,  T(-1) / 6,
                      T(-1) / 6, T(5) / 6,  T(1) / 3,  T(1) / 3,  T(-7) / 6, T(11) / 6};
    for (int q = 0; q < 12; ++q) c[q] = cc[q];
  }
}

// machine epsilon of T: epsilon(1.0_rk) in the eps check (src/hrweno_weno.f90:92)
template <class T> static T epsilon_of();
template <> float epsilon_of<float>() { return 1.1920928955078125e-07f; }
template <> double epsilon_of<double>() { return 2.220446049250313080847e-16; }

// ---------------------------------------------------------------------------------------
// weno_calc_cnu (src/hrweno_weno.f90:221-297): coefficients c(j, r, i) of Shu eq. 2.20 on
// a non-uniform grid.  xedges(0:nc); cnu stored at [j + k*(r+1) + k*(k+1)*(i-1)].
// ---------------------------------------------------------------------------------------
template <class T>
static void weno_calc_cnu(int nc, int k, const T* xedges, T* cnu) {
  const int ng = k + 1;
  // xext(0-(k+1) : nc+(k+1)), offset so that xext[q + ng] is xext(q)   (:234,241-243)
  std::vector<T> xext(nc + 2 * ng + 1);
  auto X = [&](int q) -> T& { return xext[q + ng]; };
  for (int q = 0; q <= nc; ++q) X(q) = xedges[q];
  // linear extension to the left and to the right (:245-255)
  T dx = X(1) - X(0);
  for (int q = -1; q >= -ng; --q) X(q) = X(q + 1) - dx;
  dx = X(nc) - X(nc - 1);
  for (int q = nc + 1; q <= nc + ng; ++q) X(q) = X(q - 1) + dx;
  // xl(q) = xext(q-1), xr(q) = xext(q) for q = 1-ng..   (:257-259)
  auto xl = [&](int q) { return X(q - 1); };
  auto xr = [&](int q) { return X(q); };
  for (int i = 1; i <= nc; ++i)
    for (int r = -1; r <= k - 1; ++r)
      for (int j = 0; j <= k - 1; ++j) {  // (:263-295)
        T sum2 = T(0);
        for (int m = j + 1; m <= k; ++m) {
          T prod2 = T(1);
          for (int l = 0; l <= k; ++l) {
            if (l == m) continue;
            prod2 = prod2 * (xl(i - r + m) - xl(i - r + l));
          }
          T sum1 = T(0);
          for (int l = 0; l <= k; ++l) {
            if (l == m) continue;
            T prod1 = T(1);
            for (int q = 0; q <= k; ++q) {
              if (q == m || q == l) continue;
              prod1 = prod1 * (xr(i) - xl(i - r + q));
            }
            sum1 = sum1 + prod1;
          }
          sum2 = sum2 + sum1 / prod2;
        }
        cnu[j + k * (r + 1) + k * (k + 1) * (i - 1)] = sum2 * (xr(i - r + j) - xl(i - r + j));
      }
}

// ---------------------------------------------------------------------------------------
// weno_reconstruct (src/hrweno_weno.f90:129-219), in the reference's operation order.
// cnu == nullptr selects the uniform tables.
// ---------------------------------------------------------------------------------------
template <class T>
static void weno_reconstruct(int nc, int k, T eps, const T* cnu, const T* v, T* vl, T* vr) {
  T d[3], c[12];
  tables<T>(k, d, c);
  // vext(1-(k-1) : nc+(k-1)) with constant ghosts (:163,171-173); vext[q + k - 1] = vext(q),
  // so the storage spans indices 1 .. nc + 2k - 2
  std::vector<T> vext(nc + 2 * k - 1);
  auto V = [&](int q) { return vext[q + k - 1]; };
  for (int q = 1; q <= nc; ++q) vext[q + k - 1] = v[q - 1];
  for (int q = 1 - (k - 1); q <= 0; ++q) vext[q + k - 1] = v[0];
  for (int q = nc + 1; q <= nc + k - 1; ++q) vext[q + k - 1] = v[nc - 1];
  ORC_PARFOR
  for (int i = 1; i <= nc; ++i) {  // (:174)
    const T* ci = cnu ? cnu + (size_t)k * (k + 1) * (i - 1) : c;  // (:170,177)
    auto C = [&](int j, int r) { return ci[j + k * (r + 1)]; };
    T vrr[3], vlr[3], beta[3], alfa[3], alfat[3], w[3], wt[3];
    for (int r = 0; r <= k - 1; ++r) {  // (:178-181)
      T sr = T(0), sl = T(0);
      for (int j = 0; j <= k - 1; ++j) {
        sr = sr + C(j, r) * V(i - r + j);
        sl = sl + C(j, r - 1) * V(i - r + j);
      }
      vrr[r] = sr;
      vlr[r] = sl;
    }
    if (k == 1) {  // (:185-186)
      beta[0] = T(0);
    } else if (k == 2) {  // (:189-191)
      T a = V(i + 1) - V(i), b = V(i) - V(i - 1);
      beta[0] = a * a;
      beta[1] = b * b;
    } else {  // (:194-202)
      const T c13 = T(13) / 12, c14 = T(1) / 4;
      T a, b;
      a = V(i) - 2 * V(i + 1) + V(i + 2);
      b = 3 * V(i) - 4 * V(i + 1) + V(i + 2);
      beta[0] = c13 * (a * a) + c14 * (b * b);
      a = V(i - 1) - 2 * V(i) + V(i + 1);
      b = V(i - 1) - V(i + 1);
      beta[1] = c13 * (a * a) + c14 * (b * b);
      a = V(i - 2) - 2 * V(i - 1) + V(i);
      b = V(i - 2) - 4 * V(i - 1) + 3 * V(i);
      beta[2] = c13 * (a * a) + c14 * (b * b);
    }
    for (int r = 0; r < k; ++r) {  // (:207-208)
      T e = eps + beta[r];
      alfa[r] = d[r] / (e * e);
      alfat[r] = d[k - 1 - r] / (e * e);
    }
    T sa = T(0), sat = T(0);
    for (int r = 0; r < k; ++r) { sa = sa + alfa[r]; sat = sat + alfat[r]; }
    for (int r = 0; r < k; ++r) { w[r] = alfa[r] / sa; wt[r] = alfat[r] / sat; }  // (:209-210)
    T ar = T(0), al = T(0);
    for (int r = 0; r < k; ++r) { ar = ar + w[r] * vrr[r]; al = al + wt[r] * vlr[r]; }
    vr[i - 1] = ar;  // (:213-214)
    vl[i - 1] = al;
  }
}

// ---------------------------------------------------------------------------------------
// Physical fluxes of the problem descriptor and the two monotone numerical fluxes.
// ---------------------------------------------------------------------------------------
enum { FN_TEST_UXT = 100 };  // f = u*x*t of test/test_fluxes.f90:74-78

template <class T>
static T phys_flux(int fn, T a, T b, T u, T x, T t) {
  if (fn == HRW_FN_BURGERS) return (u * u) / 2;  // example1...f90:111-122
  if (fn == FN_TEST_UXT) return u * x * t;
  if (fn == HRW_FN_BURGERS_LINEAR) return (u * u) / 2 + (a + b * x) * u;  // Burgers + g(x) u
  return (a + b * x) * u;  // f = g(x) u, example2...f90:131-155 with g = a + b x
}

// lax_friedrichs (src/hrweno_fluxes.f90:22-45, formula :43)
template <class T>
static T lax_friedrichs(int fn, T a, T b, T vm, T vp, T x, T t, T alpha) {
  return (phys_flux(fn, a, b, vm, x, t) + phys_flux(fn, a, b, vp, x, t) - alpha * (vp - vm)) / 2;
}

// godunov (src/hrweno_fluxes.f90:47-76, formula :67-74)
template <class T>
static T godunov(int fn, T a, T b, T vm, T vp, T x, T t) {
  T fm = phys_flux(fn, a, b, vm, x, t), fp = phys_flux(fn, a, b, vp, x, t);
  if (vm <= vp) return fm < fp ? fm : fp;  // min(fm, fp)
  return fm > fp ? fm : fp;                // max(fm, fp)
}

template <class T>
static T numflux(const hrw_problem& p, int dim, T vm, T vp, T x, T t) {
  if (p.flux == HRW_FLUX_GODUNOV)
    return godunov<T>(p.fn[dim], (T)p.coef_a[dim], (T)p.coef_b[dim], vm, vp, x, t);
  return lax_friedrichs<T>(p.fn[dim], (T)p.coef_a[dim], (T)p.coef_b[dim], vm, vp, x, t,
                           (T)p.alpha[dim]);
}

// ---------------------------------------------------------------------------------------
// Right-hand sides (the user `rhs` of the examples).
// ---------------------------------------------------------------------------------------
template <class T>
struct Line {  // one dimension of the grid: grid1%linear (src/hrweno_grids.f90:60-79,236-247)
  int nc = 0;
  T xmin = 0, rx = 0;
  std::vector<T> width;  // per-cell width; empty: uniform rx
  std::vector<T> edges;  // non-uniform line: edges(0:nc); empty: uniform
  std::vector<T> cnu;    // weno coefficients of the non-uniform line (weno_calc_cnu)
  T right(int i) const { return edges.empty() ? xmin + rx * (T)i : edges[i]; }  // edges(i)
  T w(int i) const { return width.empty() ? rx : width[i - 1]; }
};

// Fluxes of one line (example1...f90:93-104; example2...f90:97-120):
// F[0..nc] from v[0..nc-1] for boundary kind bc.
template <class T>
static void line_fluxes(const hrw_problem& p, int dim, const Line<T>& L, T eps, T t,
                        const T* v, T* vl, T* vr, T* F) {
  const int nc = L.nc;
  weno_reconstruct<T>(nc, p.k, eps, L.cnu.empty() ? nullptr : L.cnu.data(), v, vl, vr);
  ORC_PARFOR
  for (int i = 1; i <= nc - 1; ++i) F[i] = numflux<T>(p, dim, vr[i - 1], vl[i], L.right(i), t);
  switch (p.bc[dim]) {
    case HRW_BC_COPY:  // (example1...f90:103-104)
      if (nc >= 2) { F[0] = F[1]; F[nc] = F[nc - 1]; } else { F[0] = F[1] = T(0); }
      break;
    case HRW_BC_ZERO:  // (example2...f90:117-120)
      F[0] = T(0); F[nc] = T(0);
      break;
    default:  // ZERO_INFLOW: no inflow, outflow flux f(vr(nc)) = h(vr(nc), vr(nc))
      F[0] = T(0);
      F[nc] = phys_flux<T>(p.fn[dim], (T)p.coef_a[dim], (T)p.coef_b[dim], vr[nc - 1],
                           L.right(nc), t);
  }
}

template <class T>
struct Problem {
  hrw_problem p{};
  int neq = 0;
  Line<T> line[2];
  std::vector<T> rates;
  std::vector<T> vl, vr, F, col, vdot2;

  explicit Problem(const hrw_problem& pp, int n) : p(pp), neq(n) {
    p.width[0] = p.width[1] = nullptr;
    p.xedges[0] = p.xedges[1] = nullptr;
    p.rates = nullptr;
    int nd = pp.kind == HRW_PROBLEM_FV2D ? 2 : (pp.kind == HRW_PROBLEM_FV1D ? 1 : 0);
    for (int d = 0; d < nd; ++d) {
      Line<T>& L = line[d];
      L.nc = pp.ncells[d];
      L.xmin = (T)pp.xmin[d];
      L.rx = ((T)pp.xmax[d] - (T)pp.xmin[d]) / (T)L.nc;  // (src/hrweno_grids.f90:72)
      if (pp.width[d]) {
        L.width.resize(L.nc);
        for (int i = 0; i < L.nc; ++i) L.width[i] = (T)pp.width[d][i];
      }
      if (pp.xedges[d]) {  // weno(ncells, k, eps, xedges) and width(i) = edges(i) - edges(i-1)
        L.edges.resize(L.nc + 1);
        for (int i = 0; i <= L.nc; ++i) L.edges[i] = (T)pp.xedges[d][i];
        L.width.resize(L.nc);
        for (int i = 0; i < L.nc; ++i) L.width[i] = L.edges[i + 1] - L.edges[i];
        L.cnu.resize((size_t)pp.k * (pp.k + 1) * L.nc);
        weno_calc_cnu<T>(L.nc, pp.k, L.edges.data(), L.cnu.data());
      }
    }
    if (pp.kind == HRW_PROBLEM_LINEAR_ODE && pp.rates) {
      rates.resize(neq);
      for (int i = 0; i < neq; ++i) rates[i] = (T)pp.rates[i];
    }
    int mx = std::max(line[0].nc, line[1].nc) + 1;
    vl.resize(mx); vr.resize(mx); F.resize(mx); col.resize(mx);
  }

  void rhs(double td, const T* v, T* vdot) {
    const T t = (T)td;
    const T eps = (T)p.eps;
    if (p.kind == HRW_PROBLEM_LINEAR_ODE) {  // test/test_tvdode.f90:107-111
      for (int i = 0; i < neq; ++i) vdot[i] = rates[i] * v[i];
      return;
    }
    if (p.kind == HRW_PROBLEM_FV1D) {  // example1...f90:72-109
      const Line<T>& L = line[0];
      line_fluxes<T>(p, 0, L, eps, t, v, vl.data(), vr.data(), F.data());
      ORC_PARFOR
      for (int i = 1; i <= L.nc; ++i) vdot[i - 1] = -(F[i] - F[i - 1]) / L.w(i);  // (:107)
      return;
    }
    // FV2D (example2...f90:73-129): u((j-1)*nc1 + i), x1 fastest
    const Line<T>& L1 = line[0];
    const Line<T>& L2 = line[1];
    const int n1 = L1.nc, n2 = L2.nc;
    std::vector<T> F1((size_t)(n1 + 1) * n2), F2((size_t)(n2 + 1) * n1);
    // the rows, then the columns, split over threads (the example's own commented-out OpenMP
    // loop, example2...f90:95-114): each line's arithmetic, and so every bit, is unchanged
#ifdef _OPENMP
#pragma omp parallel
#endif
    {
      std::vector<T> tvl(vl.size()), tvr(vr.size()), tcol(col.size());
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
      for (int j = 1; j <= n2; ++j)  // x1 sweep over contiguous rows (:97-103)
        line_fluxes<T>(p, 0, L1, eps, t, v + (size_t)(j - 1) * n1, tvl.data(), tvr.data(),
                       F1.data() + (size_t)(j - 1) * (n1 + 1));
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
      for (int i = 1; i <= n1; ++i) {  // x2 sweep over strided columns (:106-112)
        for (int j = 1; j <= n2; ++j) tcol[j - 1] = v[(size_t)(j - 1) * n1 + (i - 1)];
        line_fluxes<T>(p, 1, L2, eps, t, tcol.data(), tvl.data(), tvr.data(),
                       F2.data() + (size_t)(i - 1) * (n2 + 1));
      }
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
      for (int j = 1; j <= n2; ++j)  // (:123-127)
        for (int i = 1; i <= n1; ++i) {
          const T* f1 = F1.data() + (size_t)(j - 1) * (n1 + 1);
          const T* f2 = F2.data() + (size_t)(i - 1) * (n2 + 1);
          vdot[(size_t)(j - 1) * n1 + (i - 1)] =
              -((f1[i] - f1[i - 1]) / L1.w(i)) - (f2[j] - f2[j - 1]) / L2.w(j);
        }
    }
  }
};

// ---------------------------------------------------------------------------------------
// TVD ODE integrators (src/hrweno_tvdode.f90).
// ---------------------------------------------------------------------------------------
// The time type of each build: a REAL32 build holds t, tout and dt in real32 like everything
// else (src/hrweno_kinds.F90:9-10, src/hrweno_tvdode.f90:97-135); the REAL64 build and the
// REAL128 yardstick (used for the precision of the state only) keep them in FP64.
template <class T> struct TimeOf { using type = double; };
template <> struct TimeOf<float> { using type = float; };

// is_done (src/hrweno_tvdode.f90:273-284)
template <class R>
static bool is_done(R t, R tout, R dt) {
  return (t - tout) * std::copysign(R(1), dt) > R(0);
}

template <class T>
struct ODE {
  using Time = typename TimeOf<T>::type;
  Problem<T> prob;
  int neq, order, method;  // method 0 rktvd, 1 mstvd
  int fevals = 0, istate = 0;
  long long nsteps = 0;
  std::vector<T> ui, udot, uold, udotold;  // uold(neq, 4) column-major

  ODE(const hrw_problem& p, int n, int ord, int meth) : prob(p, n), neq(n), order(ord), method(meth) {
    init();
  }
  ODE(const Problem<T>& P, int ord, int meth) : prob(P), neq(P.neq), order(ord), method(meth) {
    init();
  }
  void init() {
    ui.resize(neq); udot.resize(neq);
    if (method == 1) { uold.resize((size_t)neq * 4); udotold.resize((size_t)neq * 4); }
    istate = 1;
  }

  // one step of rktvd (src/hrweno_tvdode.f90:136-171)
  void rk_step(T* u, Time& t, Time dt, int& fe) {
    const int n = neq;
    const T dtt = (T)dt;
    if (order == 1) {  // (:137-143)
      prob.rhs(t, u, udot.data());
      ORC_PARFOR
      for (int i = 0; i < n; ++i) u[i] = u[i] + dtt * udot[i];
      fe += 1;
    } else if (order == 2) {  // (:148-155)
      prob.rhs(t, u, udot.data());
      ORC_PARFOR
      for (int i = 0; i < n; ++i) ui[i] = u[i] + dtt * udot[i];
      prob.rhs(t + dt, ui.data(), udot.data());
      ORC_PARFOR
      for (int i = 0; i < n; ++i) u[i] = (u[i] + ui[i] + dtt * udot[i]) / 2;
      fe += 2;
    } else {  // (:161-169)
      prob.rhs(t, u, udot.data());
      ORC_PARFOR
      for (int i = 0; i < n; ++i) ui[i] = u[i] + dtt * udot[i];
      prob.rhs(t + dt, ui.data(), udot.data());
      ORC_PARFOR
      for (int i = 0; i < n; ++i) ui[i] = (3 * u[i] + ui[i] + dtt * udot[i]) / 4;
      prob.rhs(t + dt / 2, ui.data(), udot.data());
      ORC_PARFOR
      for (int i = 0; i < n; ++i) u[i] = (u[i] + 2 * ui[i] + 2 * dtt * udot[i]) / 3;
      fe += 3;
    }
    t = t + dt;
    nsteps += 1;
  }

  // rktvd_integrate (src/hrweno_tvdode.f90:97-178)
  void rk_integrate(T* u, Time& t, Time tout, Time dt, int itask) {
    if (istate < 1) return;  // (:126)
    if (is_done(t, tout, dt)) return;  // (:127)
    for (;;) {
      rk_step(u, t, dt, fevals);
      if (is_done(t, tout, dt) || itask == 2) break;
    }
    if (istate == 1) istate = 2;  // (:176)
  }

  // mstvd_integrate (src/hrweno_tvdode.f90:203-271)
  void ms_integrate(T* u, Time& t, Time tout, Time dt) {
    const int n = neq;
    if (istate < 1) return;  // (:228)
    if (is_done(t, tout, dt)) return;  // (:229)
    auto UO = [&](int c) { return uold.data() + (size_t)(c - 1) * n; };     // uold(:, c)
    auto DO = [&](int c) { return udotold.data() + (size_t)(c - 1) * n; };  // udotold(:, c)
    if (istate == 1) {  // start with RK3 (:236-249)
      ODE<T> start(prob, 3, 0);  // rktvd(self%fu, neq, order) sharing the same rhs
      for (int c = order + 1; c >= 1; --c) {
        std::memcpy(UO(c), u, sizeof(T) * n);
        prob.rhs(t, u, DO(c));
        start.rk_integrate(u, t, t + 2 * dt, dt, 2);
      }
      fevals = start.fevals;  // (:246): the 4 extra rhs calls are not counted
      nsteps += start.nsteps;
      istate = 2;
    }
    const T dtt = (T)dt;
    for (;;) {  // (:252-268)
      if (is_done(t, tout, dt)) break;
      prob.rhs(t, u, udot.data());
      for (int i = 0; i < n; ++i)
        ui[i] = (25 * u[i] + 50 * dtt * udot[i] + 7 * UO(4)[i] + 10 * dtt * DO(4)[i]) / 32;
      t = t + dt;
      fevals += 1;
      nsteps += 1;
      // eoshift(..., shift=-1, dim=2): column c takes column c-1, column 1 is refilled
      for (int c = 4; c >= 2; --c) {
        std::memcpy(DO(c), DO(c - 1), sizeof(T) * n);
        std::memcpy(UO(c), UO(c - 1), sizeof(T) * n);
      }
      std::memcpy(DO(1), udot.data(), sizeof(T) * n);
      std::memcpy(UO(1), u, sizeof(T) * n);
      std::memcpy(u, ui.data(), sizeof(T) * n);
    }
  }
};

// ---------------------------------------------------------------------------------------
// Tangent-linear model: the same templates instantiated on a forward-mode dual number give the
// exact directional derivative of the discrete forward map, in the reference's operation
// order.  Comparisons (Godunov's min/max, vm <= vp) act on the value part.
// ---------------------------------------------------------------------------------------
struct Dual {
  double v = 0.0, d = 0.0;
  Dual() = default;
  Dual(double x) : v(x), d(0.0) {}  // NOLINT: implicit, like a real literal
  Dual(double x, double y) : v(x), d(y) {}
  explicit operator double() const { return v; }
};
inline Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
inline Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
inline Dual operator-(Dual a) { return {-a.v, -a.d}; }
inline Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
inline Dual operator/(Dual a, Dual b) { return {a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)}; }
inline Dual operator+(Dual a, int b) { return a + Dual(b); }
inline Dual operator*(int a, Dual b) { return Dual(a) * b; }
inline Dual operator/(Dual a, int b) { return a / Dual(b); }
inline bool operator<(Dual a, Dual b) { return a.v < b.v; }
inline bool operator>(Dual a, Dual b) { return a.v > b.v; }
inline bool operator<=(Dual a, Dual b) { return a.v <= b.v; }

struct Handle {
  int prec;
  void* ode;
};

template <class T>
static void to_T(const double* a, T* b, size_t n) { for (size_t i = 0; i < n; ++i) b[i] = (T)a[i]; }
template <class T>
static void to_D(const T* a, double* b, size_t n) { for (size_t i = 0; i < n; ++i) b[i] = (double)a[i]; }

template <class T>
static int reconstruct_T(int nc, int k, double eps, const double* xedges, const double* v,
                         double* vl, double* vr) {
  std::vector<T> tv(nc), tl(nc), tr(nc), cnu;
  to_T(v, tv.data(), nc);
  if (xedges) {
    std::vector<T> xe(nc + 1);
    to_T(xedges, xe.data(), nc + 1);
    cnu.resize((size_t)k * (k + 1) * nc);
    weno_calc_cnu<T>(nc, k, xe.data(), cnu.data());
  }
  weno_reconstruct<T>(nc, k, (T)eps, xedges ? cnu.data() : nullptr, tv.data(), tl.data(), tr.data());
  to_D(tl.data(), vl, nc);
  to_D(tr.data(), vr, nc);
  return 0;
}

template <class T>
static int integrate_T(Handle* h, double* u, double* t, double tout, double dt, int itask) {
  using Time = typename ODE<T>::Time;
  ODE<T>* o = (ODE<T>*)h->ode;
  std::vector<T> tu(o->neq);
  to_T(u, tu.data(), o->neq);
  Time tt = (Time)*t;
  if (o->method == 0) o->rk_integrate(tu.data(), tt, (Time)tout, (Time)dt, itask);
  else o->ms_integrate(tu.data(), tt, (Time)tout, (Time)dt);
  *t = (double)tt;
  to_D(tu.data(), u, o->neq);
  return 0;
}

}  // namespace orc

using namespace orc;

extern "C" {

const char* orc_last_error(void) { return g_msg.c_str(); }

// Threads used by the 1D loops (1 = the serial reference); returns the count in effect.
int orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

// weno%reconstruct at precision prec (32, 64, 128); xedges nullable (non-uniform grid).
int orc_weno_reconstruct(int prec, int nc, int k, double eps, const double* xedges,
                         const double* v, double* vl, double* vr) {
  // validation as weno_init (src/hrweno_weno.f90:72-109)
  if (nc <= 0) { g_msg = "Invalid input 'ncells'. Valid range: ncells > 0."; return HRW_EINVAL; }
  if (k < 1 || k > 3) { g_msg = "Invalid input 'k'. Valid range: 1 <= k <= 3."; return HRW_EINVAL; }
  if (prec == 32) {
    if (!((float)eps > epsilon_of<float>())) { g_msg = "Invalid input 'eps'. Valid range: eps > epsilon."; return HRW_EINVAL; }
    return reconstruct_T<float>(nc, k, eps, xedges, v, vl, vr);
  }
  if (!(eps > epsilon_of<double>())) { g_msg = "Invalid input 'eps'. Valid range: eps > epsilon."; return HRW_EINVAL; }
  if (prec == 128) return reconstruct_T<qreal>(nc, k, eps, xedges, v, vl, vr);
  return reconstruct_T<double>(nc, k, eps, xedges, v, vl, vr);
}

// weno_calc_cnu at precision 64; cnu has k*(k+1)*nc entries in Fortran order.
int orc_weno_calc_cnu(int nc, int k, const double* xedges, double* cnu) {
  if (nc <= 0 || k < 1 || k > 3) return HRW_EINVAL;
  weno_calc_cnu<double>(nc, k, xedges, cnu);
  return 0;
}

// numerical flux h(vm, vp) at (x, t): kind 0 Lax-Friedrichs, 1 Godunov; fn as HRW_FN_* or
// 100 for the test flux f = u*x*t.
double orc_numflux(int kind, int fn, double a, double b, double vm, double vp, double x,
                   double t, double alpha) {
  if (kind == HRW_FLUX_GODUNOV) return godunov<double>(fn, a, b, vm, vp, x, t);
  return lax_friedrichs<double>(fn, a, b, vm, vp, x, t, alpha);
}

// vdot = L(v) for problem p at precision prec.
int orc_rhs(int prec, const hrw_problem* p, int neq, double t, const double* v, double* vdot) {
  if (prec == 32) {
    Problem<float> P(*p, neq);
    std::vector<float> a(neq), b(neq);
    to_T(v, a.data(), neq);
    P.rhs(t, a.data(), b.data());
    to_D(b.data(), vdot, neq);
  } else if (prec == 128) {
    Problem<qreal> P(*p, neq);
    std::vector<qreal> a(neq), b(neq);
    to_T(v, a.data(), neq);
    P.rhs(t, a.data(), b.data());
    to_D(b.data(), vdot, neq);
  } else {
    Problem<double> P(*p, neq);
    P.rhs(t, v, vdot);
  }
  return 0;
}

// rktvd(fu, neq, order) (method 0) or mstvd(fu, neq) (method 1) at precision prec.
void* orc_ode_create(int prec, const hrw_problem* p, int neq, int method, int order) {
  // validation as rktvd_init / mstvd_init (src/hrweno_tvdode.f90:80-90,190-194)
  if (neq <= 0) { g_msg = "Invalid input 'neq'. Valid range: neq >= 1."; return nullptr; }
  if (method == 0 && (order < 1 || order > 3)) {
    g_msg = "Invalid input 'order' in 'rktvd'. Valid range: 1 <= k <= 3.";
    return nullptr;
  }
  if (method == 1) order = 3;
  Handle* h = new Handle;
  h->prec = prec;
  if (prec == 32) h->ode = new ODE<float>(*p, neq, order, method);
  else if (prec == 128) h->ode = new ODE<qreal>(*p, neq, order, method);
  else h->ode = new ODE<double>(*p, neq, order, method);
  return h;
}

int orc_ode_integrate(void* hh, double* u, double* t, double tout, double dt, int itask) {
  Handle* h = (Handle*)hh;
  if (h->prec == 32) return integrate_T<float>(h, u, t, tout, dt, itask);
  if (h->prec == 128) return integrate_T<qreal>(h, u, t, tout, dt, itask);
  return integrate_T<double>(h, u, t, tout, dt, itask);
}

int orc_ode_info(void* hh, int* fevals, int* istate, long long* nsteps) {
  Handle* h = (Handle*)hh;
  if (h->prec == 32) { auto o = (ODE<float>*)h->ode; *fevals = o->fevals; *istate = o->istate; *nsteps = o->nsteps; }
  else if (h->prec == 128) { auto o = (ODE<qreal>*)h->ode; *fevals = o->fevals; *istate = o->istate; *nsteps = o->nsteps; }
  else { auto o = (ODE<double>*)h->ode; *fevals = o->fevals; *istate = o->istate; *nsteps = o->nsteps; }
  return 0;
}

// J = 0.5 ||u(T) - target||^2 after nsteps rktvd(order) steps of dt from u0, and its
// directional derivative dJ = dJ/du0 . du0 by the tangent-linear (dual number) model.
int orc_tl_misfit(const hrw_problem* p, int neq, int order, const double* u0, const double* du0,
                  const double* target, double dt, long long nsteps, double* J, double* dJ) {
  ODE<Dual> ode(*p, neq, order, 0);
  std::vector<Dual> u(neq);
  for (int i = 0; i < neq; ++i) u[i] = Dual(u0[i], du0[i]);
  double t = 0.0;
  for (long long n = 0; n < nsteps; ++n) ode.rk_step(u.data(), t, dt, ode.fevals);
  double j = 0.0, dj = 0.0;
  for (int i = 0; i < neq; ++i) {
    const double r = u[i].v - target[i];
    j += 0.5 * r * r;
    dj += r * u[i].d;
  }
  *J = j;
  *dJ = dj;
  return 0;
}

void orc_ode_destroy(void* hh) {
  Handle* h = (Handle*)hh;
  if (!h) return;
  if (h->prec == 32) delete (ODE<float>*)h->ode;
  else if (h->prec == 128) delete (ODE<qreal>*)h->ode;
  else delete (ODE<double>*)h->ode;
  delete h;
}

}  // extern "C"
