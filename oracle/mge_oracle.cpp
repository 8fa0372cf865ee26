/*
 * mge_oracle.cpp -- CPU FP64 restatement of code_mge's multigrid Runge-Kutta
 * residual cycle (srcf90/solver.f90 .. srcf90/depvars.f90).
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py load this library, and only as
 * the checker.  The GPU product (code_mge_gb300) never links or calls it.
 *
 * Parity status: UNPINNED against the reference binary (Fortran, not
 * buildable here: the fcode library, plugin sources and include files are
 * absent and no Fortran compiler exists).  Every routine below restates the
 * cited Fortran routine in the same loop order and the same expression order,
 * compiled with -O2 -ffp-contract=off so that each Fortran expression rounds
 * exactly as gfortran -O2 on x86-64 (SSE2, no FMA contraction) would.
 *
 * Indexing: every per-cell array uses the Fortran layout of make_flow.f90:
 * a(0:ib,0:jb,0:kb,1:5), i fastest.  Variables are 0-based here (v = 0..4 for
 * Fortran 1..5).
 *
 * Definitions the reference takes from its absent preprocessor library and
 * that this build defines itself (they are shared with the GPU library):
 *  - uniform block metric: si = (-hy*hz,0,0), sj = (0,-hx*hz,0),
 *    sk = (0,0,-hx*hy), cellvolume = hx*hy*hz (what init_metric.f90:111-177
 *    yields for an exactly representable uniform grid);
 *  - grid transfer geometry (eval_x2cell, shft_cell, trilinear_factor): a
 *    fine block with ratio r and integer offset o inside its parent; the
 *    centre-based 2x2x2 stencil is clamped to the parent's physical cells and
 *    the local coordinate is kept unclamped (linear extrapolation);
 *  - cut-cell records and their interpolation clouds are inputs.
 */
#include "mge_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

int g_threads = 1;

struct ORec {
  int ccid[3], scid[3], faceid, zz, npoint;
  int ijk[MGE_MAX_CLOUD][3];
  double coef[MGE_MAX_CLOUD];
  double nvec[3], qb[3], area;
  double psurf[3], pnew[3];  // the surface point and its moved position (movsurf.f90:31)
  double psol, wsol[5];
};

struct OBlock {
  int level = 0, serial = 0;
  int nx = 0, ny = 0, nz = 0, il = 0, jl = 0, kl = 0, ie = 0, je = 0, ke = 0, ib = 0, jb = 0, kb = 0;
  size_t Pi = 0, Pj = 0, Pk = 0, N = 0;
  double h[3] = {0, 0, 0}, origin[3] = {0, 0, 0}, vol = 0;
  double si[3] = {0, 0, 0}, sj[3] = {0, 0, 0}, sk[3] = {0, 0, 0};
  int bctype[6] = {0, 0, 0, 0, 0, 0};
  double fnv[6][3] = {};
  std::vector<double> w, p, wn, ws, dw, fw, wr, qf, vdtim, radi, radj, radk, epsx, epsy, epsz;
  std::vector<double> w1, w2;  // states of the two previous physical time steps (execmode 1)
  std::vector<int> blank, marker;
  std::vector<double> rtrms;
  double dtim = 10.0;
  std::vector<ORec> z;
  int parent = -1, ratio[3] = {1, 1, 1}, offset[3] = {0, 0, 0};

  inline size_t I(int i, int j, int k) const { return (size_t)i + Pi * ((size_t)j + Pj * (size_t)k); }
  inline double& W(int i, int j, int k, int v) { return w[(size_t)v * N + I(i, j, k)]; }
  inline double& P(int i, int j, int k) { return p[I(i, j, k)]; }
  inline double& DW(int i, int j, int k, int v) { return dw[(size_t)v * N + I(i, j, k)]; }
  inline double& FW(int i, int j, int k, int v) { return fw[(size_t)v * N + I(i, j, k)]; }
  inline int BL(int i, int j, int k) const { return blank[I(i, j, k)]; }
  inline double LAM(int i, int j, int k) const {
    size_t c = I(i, j, k);
    return radi[c] + radj[c] + radk[c];
  }
};

}  // namespace

struct mgeo_ctx {
  mge_params prm;
  std::vector<std::vector<OBlock>> lv;  // lv[level-1][serial-1]
  std::string err;
  bool committed = false;
  int mirr_zero_warned = 0;
  int itime = 0;  // physical time step counter of the unsteady mode (solver.f90:115,286)
};

namespace {

inline double fdim_(double a, double b) { return a > b ? a - b : 0.0; }  // Fortran DIM
inline double fmax_(double a, double b) { return a > b ? a : b; }
inline double fmin_(double a, double b) { return a < b ? a : b; }

int fail(mgeo_ctx* c, int code, const std::string& msg) {
  c->err = msg;
  return code;
}

OBlock* getb(mgeo_ctx* c, int level, int serial) {
  if (level < 1 || level > (int)c->lv.size()) return nullptr;
  auto& L = c->lv[level - 1];
  if (serial < 1 || serial > (int)L.size()) return nullptr;
  return &L[serial - 1];
}

/* depvars_one, depvars.f90:48-49:  qq = 0.5*sum(cv(2:4)**2)/cv(1); p = (g-1)*dim(cv(5),qq) */
inline double depvars_one(const double gamma, double w0, double w1, double w2, double w3, double w4) {
  double qq = 0.5 * (w1 * w1 + w2 * w2 + w3 * w3) / w0;
  return (gamma - 1.0) * fdim_(w4, qq);
}

void depvars_cell(const mge_params& P, OBlock& b, int i, int j, int k) {
  b.P(i, j, k) = depvars_one(P.gamma, b.W(i, j, k, 0), b.W(i, j, k, 1), b.W(i, j, k, 2), b.W(i, j, k, 3),
                             b.W(i, j, k, 4));
}

/* depvars_all, depvars.f90:23-32 over the whole array 0:ib,0:jb,0:kb */
void depvars_all(const mge_params& P, OBlock& b) {
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 0; k <= b.kb; k++)
    for (int j = 0; j <= b.jb; j++)
      for (int i = 0; i <= b.ib; i++) depvars_cell(P, b, i, j, k);
}

/* ceflux, eflux.f90:133-155 / ceflux.f90:18-22 */
inline void ceflux(const double* w, double p, const double* ss, double* fs) {
  fs[0] = w[1] * ss[0] + w[2] * ss[1] + w[3] * ss[2];
  fs[1] = fs[0] * w[1] / w[0] + p * ss[0];
  fs[2] = fs[0] * w[2] / w[0] + p * ss[1];
  fs[3] = fs[0] * w[3] / w[0] + p * ss[2];
  fs[4] = fs[0] * (w[4] + p) / w[0];
}

inline void getw(OBlock& b, int i, int j, int k, double* o) {
  for (int v = 0; v < 5; v++) o[v] = b.W(i, j, k, v);
}

/* ------------------------------------------------------------------ timestep.f90 */
int timestep(mgeo_ctx* c, OBlock& b) {
  const mge_params& P = c->prm;
  const double gamma = P.gamma, cfl = P.cfl;
  const double plim = 0.001;
  const int i2d = 0;
  b.dtim = 10.0;  // timestep.f90:36
  double cfac = 4.0;
  if (P.eqntype == MGE_EQN_NS) {
    if (P.distype == MGE_DIS_CENTRAL) cfac = 4.0;       // timestep.f90:119-125
    else if (P.distype == MGE_DIS_ROE2) cfac = 1.0;
    else cfac = 2.0;
  }
  const bool ns = (P.eqntype == MGE_EQN_NS);
  int bad = 0;
  double dtmin = 10.0;
#pragma omp parallel for num_threads(g_threads) schedule(static) reduction(min : dtmin) reduction(+ : bad)
  for (int k = 2; k <= b.kl; k++)
    for (int j = 2; j <= b.jl; j++)
      for (int i = 2; i <= b.il; i++) {
        double w0 = b.W(i, j, k, 0);
        double cc = gamma * b.P(i, j, k) / w0;
        if (cc < 0.0 || cc != cc) {  // timestep.f90:45-48 (stop)
          bad++;
          continue;
        }
        cc = std::sqrt(fmax_(cc, 0.0));
        double uu = b.W(i, j, k, 1) / w0;
        double uv = b.W(i, j, k, 2) / w0;
        double uw = b.W(i, j, k, 3) / w0;
        double dtv = 0.0;
        if (ns) {  // timestep.f90:141-145
          double fmue = P.viscl / P.prlmean;
          double f1 = 4.0 / w0 / 3.0;
          double f2 = gamma / w0;
          double fac = fmax_(f1, f2);
          dtv = fac * fmue / b.vol;
        }
        double sx, sy, sz, qs, ds, cs;
        sx = 0.5 * (b.si[0] + b.si[0]);
        sy = 0.5 * (b.si[1] + b.si[1]);
        sz = 0.5 * (b.si[2] + b.si[2]);
        qs = std::fabs(uu * sx + uv * sy + uw * sz);
        ds = sx * sx + sy * sy + sz * sz;
        cs = cc * std::sqrt(ds);
        double ri = qs + cs, rvi = dtv * ds;
        sx = 0.5 * (b.sj[0] + b.sj[0]);
        sy = 0.5 * (b.sj[1] + b.sj[1]);
        sz = 0.5 * (b.sj[2] + b.sj[2]);
        qs = std::fabs(uu * sx + uv * sy + uw * sz);
        ds = sx * sx + sy * sy + sz * sz;
        cs = cc * std::sqrt(ds);
        double rj = qs + cs, rvj = dtv * ds;
        sx = 0.5 * (b.sk[0] + b.sk[0]);
        sy = 0.5 * (b.sk[1] + b.sk[1]);
        sz = 0.5 * (b.sk[2] + b.sk[2]);
        qs = std::fabs(uu * sx + uv * sy + uw * sz);
        ds = sx * sx + sy * sy + sz * sz;
        cs = cc * std::sqrt(ds);
        double rk = qs + cs, rvk = dtv * ds;
        size_t cidx = b.I(i, j, k);
        b.radi[cidx] = ri;
        b.radj[cidx] = rj;
        b.radk[cidx] = rk;
        double fict;
        if (ns)
          fict = b.vol / (ri + rj + rk + cfac * (rvi + rvj + rvk));  // timestep.f90:177-178
        else
          fict = b.vol / (ri + rj + rk);  // timestep.f90:85
        // timestep.f90:85-99 (and 180-190 for NS): the steady local step, or
        // in the unsteady mode at most 2*dtstep/(3*cfl)
        double vd = fict;
        if (P.execmode == 1) {
          const double dtime = 2.0 * P.dtstep / (3.0 * P.cfl);
          vd = fmin_(fict, dtime);
        }
        double pc = b.P(i, j, k);
        double pip = b.P(i + 1, j, k), pim = b.P(i - 1, j, k);
        double pjp = b.P(i, j + 1, k), pjm = b.P(i, j - 1, k);
        double pkp = b.P(i, j, k + 1), pkm = b.P(i, j, k - 1);
        double dpi = std::fabs((pip - 2.0 * pc + pim) / (pip + 2.0 * pc + pim + plim));
        double dpj = std::fabs((pjp - 2.0 * pc + pjm) / (pjp + 2.0 * pc + pjm + plim));
        double dpk = std::fabs((pkp - 2.0 * pc + pkm) / (pkp + 2.0 * pc + pkm + plim));
        double r = 1.0 / (1.0 + fmin_(fdim_(cfl, 1.0), 2.0 * (dpi + dpj + dpk * (1.0 - i2d))));
        vd = vd * r;  // timestep.f90:108-109
        b.vdtim[cidx] = vd;
        if (vd < dtmin) dtmin = vd;  // timestep.f90:112
      }
  if (bad) return fail(c, MGE_ENEGPRESS, "timestep: negative or NaN c^2 (timestep.f90:45-48)");
  b.dtim = dtmin;
  // zero blanked cells, timestep.f90:212-223
  for (size_t q = 0; q < b.N; q++)
    if (b.blank[q] == 0) {
      b.vdtim[q] = 0.0;
      b.radi[q] = 0.0;
      b.radj[q] = 0.0;
      b.radk[q] = 0.0;
    }
  // ghost copies, timestep.f90:227-282
  std::vector<double>* R[3] = {&b.radi, &b.radj, &b.radk};
  for (int i = 0; i <= b.ib; i++)
    for (int j = 0; j <= b.jb; j++)
      for (int t = 0; t < 3; t++) {
        std::vector<double>& a = *R[t];
        a[b.I(i, j, 0)] = a[b.I(i, j, 2)];
        a[b.I(i, j, 1)] = a[b.I(i, j, 2)];
        a[b.I(i, j, b.ke)] = a[b.I(i, j, b.kl)];
        a[b.I(i, j, b.kb)] = a[b.I(i, j, b.kl)];
      }
  for (int j = 2; j <= b.jl; j++)
    for (int k = 0; k <= b.kb; k++)
      for (int t = 0; t < 3; t++) {
        std::vector<double>& a = *R[t];
        a[b.I(0, j, k)] = a[b.I(2, j, k)];
        a[b.I(1, j, k)] = a[b.I(2, j, k)];
        a[b.I(b.ie, j, k)] = a[b.I(b.il, j, k)];
        a[b.I(b.ib, j, k)] = a[b.I(b.il, j, k)];
      }
  for (int i = 2; i <= b.il; i++)
    for (int k = 2; k <= b.kl; k++)
      for (int t = 0; t < 3; t++) {
        std::vector<double>& a = *R[t];
        a[b.I(i, 0, k)] = a[b.I(i, 2, k)];
        a[b.I(i, 1, k)] = a[b.I(i, 2, k)];
        a[b.I(i, b.je, k)] = a[b.I(i, b.jl, k)];
        a[b.I(i, b.jb, k)] = a[b.I(i, b.jl, k)];
      }
  // IRS coefficients, timestep.f90:286-309 (used only by the psmoo variant).
  // min/max follow the NaN-ignoring fmin/fmax convention (0/0 at blanked cells).
  if (P.smoo > 0.0) {
    double cflrat = std::sqrt(1.0 + 4.0 * P.smoo);
    for (int k = 2; k <= b.kl; k++)
      for (int j = 2; j <= b.jl; j++)
        for (int i = 2; i <= b.il; i++) {
          size_t q = b.I(i, j, k);
          double ri = b.radi[q], rj = b.radj[q], rk = b.radk[q];
          double reval, ex, t;
          reval = rj / ri + rk / ri;
          t = cflrat / (1.0 + 0.0625 * reval);
          ex = 0.25 * (t * t - 1.0);
          ex = std::fmin(P.smoo, ex);
          b.epsx[q] = std::fmax(0.0, ex);
          reval = rk / rj + ri / rj;
          t = cflrat / (1.0 + 0.0625 * reval);
          ex = 0.25 * (t * t - 1.0);
          ex = std::fmin(P.smoo, ex);
          b.epsy[q] = std::fmax(0.0, ex);
          reval = ri / rk + rj / rk;
          t = cflrat / (1.0 + 0.0625 * reval);
          ex = 0.25 * (t * t - 1.0);
          ex = std::fmin(P.smoo, ex);
          b.epsz[q] = std::fmax(0.0, ex);
        }
  }
  return MGE_OK;
}

/* ------------------------------------------------------------------ eflux.f90 + efluxb.f90 */
int eflux(mgeo_ctx* c, OBlock& b) {
  const size_t N = b.N;
  std::vector<double> efsx(5 * N, 0.0), efsy(5 * N, 0.0), efsz(5 * N, 0.0);
  // i-direction, eflux.f90:42-58
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 2; k <= b.kl; k++)
    for (int j = 2; j <= b.jl; j++)
      for (int i = 2; i <= b.ie; i++) {
        double w1[5], w2[5], f1[5], f2[5];
        getw(b, i, j, k, w1);
        getw(b, i - 1, j, k, w2);
        ceflux(w1, b.P(i, j, k), b.si, f1);
        ceflux(w2, b.P(i - 1, j, k), b.si, f2);
        for (int v = 0; v < 5; v++) efsx[v * N + b.I(i, j, k)] = 0.5 * (f1[v] + f2[v]);
      }
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 2; k <= b.kl; k++)
    for (int j = 2; j <= b.jl; j++)
      for (int i = 2; i <= b.il; i++)
        for (int v = 0; v < 5; v++)
          b.DW(i, j, k, v) = efsx[v * N + b.I(i, j, k)] - efsx[v * N + b.I(i + 1, j, k)];
  // j-direction (i2d == 0 always, input_param.f90:42), eflux.f90:61-79
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 2; k <= b.kl; k++)
    for (int j = 2; j <= b.je; j++)
      for (int i = 2; i <= b.il; i++) {
        double w1[5], w2[5], f1[5], f2[5];
        getw(b, i, j, k, w1);
        getw(b, i, j - 1, k, w2);
        ceflux(w1, b.P(i, j, k), b.sj, f1);
        ceflux(w2, b.P(i, j - 1, k), b.sj, f2);
        for (int v = 0; v < 5; v++) efsy[v * N + b.I(i, j, k)] = 0.5 * (f1[v] + f2[v]);
      }
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 2; k <= b.kl; k++)
    for (int j = 2; j <= b.jl; j++)
      for (int i = 2; i <= b.il; i++)
        for (int v = 0; v < 5; v++)
          b.DW(i, j, k, v) = b.DW(i, j, k, v) + efsy[v * N + b.I(i, j, k)] - efsy[v * N + b.I(i, j + 1, k)];
  // k-direction, eflux.f90:82-98
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 2; k <= b.ke; k++)
    for (int j = 2; j <= b.jl; j++)
      for (int i = 2; i <= b.il; i++) {
        double w1[5], w2[5], f1[5], f2[5];
        getw(b, i, j, k, w1);
        getw(b, i, j, k - 1, w2);
        ceflux(w1, b.P(i, j, k), b.sk, f1);
        ceflux(w2, b.P(i, j, k - 1), b.sk, f2);
        for (int v = 0; v < 5; v++) efsz[v * N + b.I(i, j, k)] = 0.5 * (f1[v] + f2[v]);
      }
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 2; k <= b.kl; k++)
    for (int j = 2; j <= b.jl; j++)
      for (int i = 2; i <= b.il; i++)
        for (int v = 0; v < 5; v++)
          b.DW(i, j, k, v) = b.DW(i, j, k, v) + efsz[v * N + b.I(i, j, k)] - efsz[v * N + b.I(i, j, k + 1)];

  // efluxb.f90:30-114, records in order
  for (size_t m = 0; m < b.z.size(); m++) {
    ORec& t = b.z[m];
    int id = t.faceid, zz = t.zz;
    int i = t.ccid[0], j = t.ccid[1], k = t.ccid[2];
    const double* sc = zz == 1 ? b.si : (zz == 2 ? b.sj : b.sk);  // uniform block: si(icut) == si(isol)
    const double* ss = sc;
    if (std::fabs(b.W(i, j, k, 0)) < 1.0e-8)  // efluxb.f90:61-64
      return fail(c, MGE_EZERORHO, "efluxb: zero density at a cut cell (efluxb.f90:61-64)");
    double wc[5], f1[5], f2[5], f3[5], fs[5], fa[5], wn[5];
    getw(b, i, j, k, wc);
    ceflux(wc, b.P(i, j, k), sc, f1);
    ceflux(t.wsol, t.psol, ss, f2);
    for (int v = 0; v < 5; v++) fs[v] = 0.5 * (f1[v] + f2[v]);
    std::vector<double>* E = zz == 1 ? &efsx : (zz == 2 ? &efsy : &efsz);
    int di = zz == 1, dj = zz == 2, dk = zz == 3;
    for (int v = 0; v < 5; v++)
      b.DW(i, j, k, v) = b.DW(i, j, k, v) - ((*E)[v * N + b.I(i, j, k)] - (*E)[v * N + b.I(i + di, j + dj, k + dk)]);
    if (id == 4 || id == 5 || id == 6) {  // solid on the + side: keep the - face
      getw(b, i - di, j - dj, k - dk, wn);
      ceflux(wn, b.P(i - di, j - dj, k - dk), sc, f3);
      for (int v = 0; v < 5; v++) {
        fa[v] = 0.5 * (f1[v] + f3[v]);
        b.DW(i, j, k, v) = b.DW(i, j, k, v) + fa[v] - fs[v];
      }
    } else if (id == 1 || id == 2 || id == 3) {  // solid on the - side: keep the + face
      getw(b, i + di, j + dj, k + dk, wn);
      ceflux(wn, b.P(i + di, j + dj, k + dk), sc, f3);
      for (int v = 0; v < 5; v++) {
        fa[v] = 0.5 * (f1[v] + f3[v]);
        b.DW(i, j, k, v) = b.DW(i, j, k, v) + fs[v] - fa[v];
      }
    }
  }
  return MGE_OK;
}

/* dflux_matrix, dflux.f90:283-339 (ff may alias dw, as in dfluxb) */
void dflux_matrix(double gamma, const double* u1, const double* u2, const double* dw, const double* ss,
                  double* ff) {
  double gam1 = gamma - 1.0, epsn = 1.0, epsl = 1.0;
  double rr = 0.5 * (u1[0] + u2[0]);
  double us[3];
  for (int q = 0; q < 3; q++) us[q] = 0.5 * (u1[q + 1] + u2[q + 1]) / rr;
  double ee = 0.5 * (u1[4] + u2[4]) / rr;
  double qq = 0.5 * (us[0] * us[0] + us[1] * us[1] + us[2] * us[2]);
  double c2 = gamma * gam1 * (ee - qq);
  double hh = c2 / gam1 + qq;
  double sss = ss[0] * ss[0] + ss[1] * ss[1] + ss[2] * ss[2];
  double cs = std::sqrt(c2 * sss);
  double qn = ss[0] * us[0] + ss[1] * us[1] + ss[2] * us[2];
  double e0 = std::fabs(qn) + cs;
  double e1 = fmax_(epsn * e0, std::fabs(qn + cs));
  double e2 = fmax_(epsn * e0, std::fabs(qn - cs));
  double e3 = fmax_(epsl * e0, std::fabs(qn));
  double s1 = 0.5 * (e1 + e2), s2 = 0.5 * (e1 - e2), s3 = e3;
  double ak1 = (s1 - s3) / c2 * gam1;
  double ak2 = s2 / cs;
  double ak3 = c2 / gam1 / sss;
  double d0 = dw[0], d1 = dw[1], d2 = dw[2], d3 = dw[3], d4 = dw[4];
  double vd = qq * d0 - us[0] * d1 - us[1] * d2 - us[2] * d3 + d4;
  double qd = qn * d0 - ss[0] * d1 - ss[1] * d2 - ss[2] * d3;
  ff[0] = ak1 * vd - ak2 * qd + s3 * d0;
  ff[1] = ak1 * (us[0] * vd - ss[0] * ak3 * qd) + ak2 * (gam1 * ss[0] * vd - us[0] * qd) + s3 * d1;
  ff[2] = ak1 * (us[1] * vd - ss[1] * ak3 * qd) + ak2 * (gam1 * ss[1] * vd - us[1] * qd) + s3 * d2;
  ff[3] = ak1 * (us[2] * vd - ss[2] * ak3 * qd) + ak2 * (gam1 * ss[2] * vd - us[2] * qd) + s3 * d3;
  ff[4] = ak1 * (hh * vd - qn * ak3 * qd) + ak2 * (gam1 * qn * vd - hh * qd) + s3 * d4;
}

/* dfluxb.f90:29-423 for one record; w(:,5) holds the enthalpy while called */
void dfluxb_rec(mgeo_ctx* c, OBlock& b, int istage, const ORec& t, const std::vector<double>& dfsx,
                const std::vector<double>& dfsy, const std::vector<double>& dfsz) {
  const mge_params& P = c->prm;
  const size_t N = b.N;
  const double cd = P.cdis[istage - 1];
  const bool scalar = P.dissip == MGE_DISSIP_SCALAR;
  int id = t.faceid, zz = t.zz;
  int i = t.ccid[0], j = t.ccid[1], k = t.ccid[2];
  double psol = t.psol;
  double wsol[5];
  for (int v = 0; v < 5; v++) wsol[v] = t.wsol[v];
  wsol[4] = wsol[4] + psol;  // dfluxb.f90:38
  double fp[3], ep, lm, lp, lam, dis2, dis4;
  double diw[3][5], fs1[5], fs2[5];
  auto pp = [&](int a) -> double {  // p along the record axis at offset a from the cut cell
    return zz == 1 ? b.P(i + a, j, k) : (zz == 2 ? b.P(i, j + a, k) : b.P(i, j, k + a));
  };
  auto ww = [&](int a, int v) -> double {
    return zz == 1 ? b.W(i + a, j, k, v) : (zz == 2 ? b.W(i, j + a, k, v) : b.W(i, j, k + a, v));
  };
  auto lamc = [&](int a) -> double {
    return zz == 1 ? b.LAM(i + a, j, k) : (zz == 2 ? b.LAM(i, j + a, k) : b.LAM(i, j, k + a));
  };
  const std::vector<double>& D = zz == 1 ? dfsx : (zz == 2 ? dfsy : dfsz);
  auto dd = [&](int a, int v) -> double {
    size_t q = zz == 1 ? b.I(i + a, j, k) : (zz == 2 ? b.I(i, j + a, k) : b.I(i, j, k + a));
    return D[v * N + q];
  };
  auto fwr = [&](int a, int v) -> double& {
    size_t q = zz == 1 ? b.I(i + a, j, k) : (zz == 2 ? b.I(i, j + a, k) : b.I(i, j, k + a));
    return b.fw[v * N + q];
  };
  const double* s_lo = zz == 1 ? b.si : (zz == 2 ? b.sj : b.sk);  // uniform: s(i) == s(i+1)
  const int lim = zz == 1 ? b.ib : (zz == 2 ? b.jb : b.kb);
  const int pos = zz == 1 ? i : (zz == 2 ? j : k);
  auto setdis = [&]() {
    dis2 = P.vis2 * ep;
    dis4 = P.vis4;
    dis4 = fdim_(dis4, dis2);
    dis2 = dis2 * cd;
    dis4 = dis4 * cd;
  };
  if (id == 4 || id == 5 || id == 6) {
    for (int v = 0; v < 5; v++) {
      fwr(0, v) = fwr(0, v) - (dd(0, v) - dd(1, v));
      fwr(-1, v) = fwr(-1, v) - (dd(-1, v) - dd(0, v));
    }
    // the three axes write the same sensors with different operand orders
    if (zz == 1) {
      fp[0] = std::fabs(pp(-2) - 2.0 * pp(-1) + pp(0)) / std::fabs(pp(-2) + 2.0 * pp(-1) + pp(0));
      fp[1] = std::fabs(pp(-1) - 2.0 * pp(0) + psol) / std::fabs(pp(-1) + 2.0 * pp(0) + psol);
    } else {
      fp[0] = std::fabs(pp(0) - 2.0 * pp(-1) + pp(-2)) / std::fabs(pp(0) + 2.0 * pp(-1) + pp(-2));
      fp[1] = std::fabs(psol - 2.0 * pp(0) + pp(-1)) / std::fabs(psol + 2.0 * pp(0) + pp(-1));
    }
    ep = fmax_(fp[0], fp[1]);
    lm = lamc(0);
    lam = lm;
    setdis();
    for (int v = 0; v < 5; v++) {
      diw[0][v] = ww(0, v) - ww(-1, v);
      diw[1][v] = wsol[v] - ww(0, v);
      diw[2][v] = diw[1][v];
      fs2[v] = diw[2][v] - 2.0 * diw[1][v] + diw[0][v];
      fs2[v] = dis2 * diw[1][v] - dis4 * fs2[v];
    }
    if (scalar) {
      for (int v = 0; v < 5; v++) fs2[v] = fs2[v] * lam;
    } else {
      double wc[5];
      for (int v = 0; v < 5; v++) wc[v] = ww(0, v);
      dflux_matrix(P.gamma, wc, wsol, fs2, s_lo, fs2);
    }
    if (pos - 3 >= 0)
      fp[2] = std::fabs(pp(-1) - 2.0 * pp(-2) + pp(-3)) / std::fabs(pp(-1) + 2.0 * pp(-2) + pp(-3));
    else
      fp[2] = 0.0;
    ep = fmax_(fmax_(fp[0], fp[1]), fp[2]);
    lm = lamc(-1);
    lp = lamc(0);
    lam = 0.5 * (lm + lp);
    setdis();
    for (int v = 0; v < 5; v++) {
      diw[0][v] = ww(-1, v) - ww(-2, v);
      diw[1][v] = ww(0, v) - ww(-1, v);
      diw[2][v] = wsol[v] - ww(0, v);
      fs1[v] = diw[2][v] - 2.0 * diw[1][v] + diw[0][v];
      fs1[v] = dis2 * diw[1][v] - dis4 * fs1[v];
    }
    if (scalar) {
      for (int v = 0; v < 5; v++) fs1[v] = fs1[v] * lam;
    } else {
      double wa[5], wc[5];
      for (int v = 0; v < 5; v++) {
        wa[v] = ww(-1, v);
        wc[v] = ww(0, v);
      }
      dflux_matrix(P.gamma, wa, wc, fs1, s_lo, fs1);
    }
    for (int v = 0; v < 5; v++) {
      fwr(0, v) = fwr(0, v) + (fs1[v] - fs2[v]);
      fwr(-1, v) = fwr(-1, v) + (dd(-1, v) - fs1[v]);
    }
  } else if (id == 1 || id == 2 || id == 3) {
    for (int v = 0; v < 5; v++) {
      fwr(0, v) = fwr(0, v) - (dd(0, v) - dd(1, v));
      fwr(1, v) = fwr(1, v) - (dd(1, v) - dd(2, v));
    }
    fp[0] = std::fabs(pp(1) - 2.0 * pp(0) + psol) / std::fabs(pp(1) + 2.0 * pp(0) + psol);
    fp[1] = std::fabs(pp(2) - 2.0 * pp(1) + pp(0)) / std::fabs(pp(2) + 2.0 * pp(1) + pp(0));
    if (pos + 3 <= lim)
      fp[2] = std::fabs(pp(3) - 2.0 * pp(2) + pp(1)) / std::fabs(pp(3) + 2.0 * pp(2) + pp(1));
    else
      fp[2] = 0.0;
    ep = fmax_(fmax_(fp[0], fp[1]), fp[2]);
    lm = lamc(0);
    lp = lamc(1);
    lam = 0.5 * (lm + lp);
    setdis();
    for (int v = 0; v < 5; v++) {
      diw[0][v] = ww(0, v) - wsol[v];
      diw[1][v] = ww(1, v) - ww(0, v);
      diw[2][v] = ww(2, v) - ww(1, v);
      fs2[v] = diw[2][v] - 2.0 * diw[1][v] + diw[0][v];
      fs2[v] = dis2 * diw[1][v] - dis4 * fs2[v];
    }
    if (scalar) {
      for (int v = 0; v < 5; v++) fs2[v] = fs2[v] * lam;
    } else {
      double wc[5], wb[5];
      for (int v = 0; v < 5; v++) {
        wc[v] = ww(0, v);
        wb[v] = ww(1, v);
      }
      dflux_matrix(P.gamma, wc, wb, fs2, s_lo, fs2);
    }
    ep = fmax_(fp[0], fp[1]);
    lp = lamc(0);
    lam = lp;
    setdis();
    for (int v = 0; v < 5; v++) {
      diw[1][v] = ww(0, v) - wsol[v];
      diw[0][v] = diw[1][v];
      diw[2][v] = ww(1, v) - ww(0, v);
      fs1[v] = diw[2][v] - 2.0 * diw[1][v] + diw[0][v];
      fs1[v] = dis2 * diw[1][v] - dis4 * fs1[v];
    }
    if (scalar) {
      for (int v = 0; v < 5; v++) fs1[v] = fs1[v] * lam;
    } else {
      double wc[5];
      for (int v = 0; v < 5; v++) wc[v] = ww(0, v);
      dflux_matrix(P.gamma, wsol, wc, fs1, s_lo, fs1);
    }
    for (int v = 0; v < 5; v++) {
      fwr(0, v) = fwr(0, v) + (fs1[v] - fs2[v]);
      fwr(1, v) = fwr(1, v) + (fs2[v] - dd(2, v));
    }
  }
}

/* ------------------------------------------------------------------ dflux.f90:1-281 */
int dflux(mgeo_ctx* c, OBlock& b, int istage) {
  const mge_params& P = c->prm;
  const double cd = P.cdis[istage - 1];
  if (cd <= 0.0) return MGE_OK;
  const bool scalar = P.dissip == MGE_DISSIP_SCALAR;
  if (P.dissip != MGE_DISSIP_SCALAR && P.dissip != MGE_DISSIP_MATRIX)
    return fail(c, MGE_EBADCFG, "dissip must be scalar or matrix (dflux.f90:107)");
  const size_t N = b.N;
  const int mx = std::max(b.ib, std::max(b.jb, b.kb));
  std::vector<double> dfsx(5 * N, 0.0), dfsy(5 * N, 0.0), dfsz(5 * N, 0.0), we(N);
  // replace energy by enthalpy, dflux.f90:58-65
  for (size_t q = 0; q < N; q++) {
    we[q] = b.w[4 * N + q];
    b.w[4 * N + q] = b.w[4 * N + q] + b.p[q];
  }
  auto face = [&](double ep, double lm, double lp, const double* dm, const double* d0, const double* dp1,
                  const double* wl, const double* wr, const double* ss, double* out) {
    double lam = 0.5 * (lm + lp);
    double dis2 = P.vis2 * ep;
    double dis4 = P.vis4;
    dis4 = fdim_(dis4, dis2);
    dis2 = dis2 * cd;
    dis4 = dis4 * cd;
    for (int v = 0; v < 5; v++) {
      double t = dp1[v] - 2.0 * d0[v] + dm[v];
      out[v] = dis2 * d0[v] - dis4 * t;
    }
    if (scalar) {
      for (int v = 0; v < 5; v++) out[v] = out[v] * lam;
    } else {
      double fs[5];
      dflux_matrix(P.gamma, wl, wr, out, ss, fs);
      for (int v = 0; v < 5; v++) out[v] = fs[v];
    }
  };
  // i-direction, dflux.f90:68-124
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 2; k <= b.kl; k++)
    for (int j = 2; j <= b.jl; j++) {
      std::vector<double> fp(mx + 1, 0.0), diw((mx + 1) * 5, 0.0);
      for (int i = 1; i <= b.ie; i++) {
        double pb = std::fabs(b.P(i - 1, j, k) + 2.0 * b.P(i, j, k) + b.P(i + 1, j, k));
        if (std::fabs(pb) > 0.0)
          fp[i] = std::fabs(b.P(i - 1, j, k) - 2.0 * b.P(i, j, k) + b.P(i + 1, j, k)) / pb;
        else
          fp[i] = 0.0;
      }
      fp[0] = 0.0;
      fp[b.ib] = 0.0;
      for (int i = 2; i <= b.ie; i++)
        for (int v = 0; v < 5; v++) diw[i * 5 + v] = b.W(i, j, k, v) - b.W(i - 1, j, k, v);
      for (int v = 0; v < 5; v++) {
        diw[1 * 5 + v] = diw[2 * 5 + v];
        diw[b.ib * 5 + v] = diw[b.ie * 5 + v];
      }
      for (int i = 2; i <= b.ie; i++) {
        double ep = fmax_(fmax_(fmax_(fp[i - 2], fp[i - 1]), fp[i]), fp[i + 1]);
        double out[5], wl[5], wr[5];
        getw(b, i - 1, j, k, wl);
        getw(b, i, j, k, wr);
        face(ep, b.LAM(i - 1, j, k), b.LAM(i, j, k), &diw[(i - 1) * 5], &diw[i * 5], &diw[(i + 1) * 5], wl, wr,
             b.si, out);
        for (int v = 0; v < 5; v++) dfsx[v * N + b.I(i, j, k)] = out[v];
      }
    }
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 2; k <= b.kl; k++)
    for (int j = 2; j <= b.jl; j++)
      for (int i = 2; i <= b.il; i++)
        for (int v = 0; v < 5; v++)
          b.FW(i, j, k, v) = b.FW(i, j, k, v) + (dfsx[v * N + b.I(i, j, k)] - dfsx[v * N + b.I(i + 1, j, k)]);
  // j-direction, dflux.f90:127-182
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 2; k <= b.kl; k++)
    for (int i = 2; i <= b.il; i++) {
      std::vector<double> fp(mx + 1, 0.0), diw((mx + 1) * 5, 0.0);
      for (int j = 1; j <= b.je; j++) {
        double pb = std::fabs(b.P(i, j + 1, k) + 2.0 * b.P(i, j, k) + b.P(i, j - 1, k));
        if (std::fabs(pb) > 0.0)
          fp[j] = std::fabs(b.P(i, j + 1, k) - 2.0 * b.P(i, j, k) + b.P(i, j - 1, k)) / pb;
        else
          fp[j] = 0.0;
      }
      fp[0] = 0.0;
      fp[b.jb] = 0.0;
      for (int j = 2; j <= b.je; j++)
        for (int v = 0; v < 5; v++) diw[j * 5 + v] = b.W(i, j, k, v) - b.W(i, j - 1, k, v);
      for (int v = 0; v < 5; v++) {
        diw[1 * 5 + v] = diw[2 * 5 + v];
        diw[b.jb * 5 + v] = diw[b.je * 5 + v];
      }
      for (int j = 2; j <= b.je; j++) {
        double ep = fmax_(fmax_(fmax_(fp[j - 2], fp[j - 1]), fp[j]), fp[j + 1]);
        double out[5], wl[5], wr[5];
        getw(b, i, j - 1, k, wl);
        getw(b, i, j, k, wr);
        face(ep, b.LAM(i, j - 1, k), b.LAM(i, j, k), &diw[(j - 1) * 5], &diw[j * 5], &diw[(j + 1) * 5], wl, wr,
             b.sj, out);
        for (int v = 0; v < 5; v++) dfsy[v * N + b.I(i, j, k)] = out[v];
      }
    }
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 2; k <= b.kl; k++)
    for (int j = 2; j <= b.jl; j++)
      for (int i = 2; i <= b.il; i++)
        for (int v = 0; v < 5; v++)
          b.FW(i, j, k, v) = b.FW(i, j, k, v) + (dfsy[v * N + b.I(i, j, k)] - dfsy[v * N + b.I(i, j + 1, k)]);
  // k-direction, dflux.f90:185-238
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int i = 2; i <= b.il; i++)
    for (int j = 2; j <= b.jl; j++) {
      std::vector<double> fp(mx + 1, 0.0), diw((mx + 1) * 5, 0.0);
      for (int k = 1; k <= b.ke; k++) {
        double pb = std::fabs(b.P(i, j, k - 1) + 2.0 * b.P(i, j, k) + b.P(i, j, k + 1));
        if (std::fabs(pb) > 0.0)
          fp[k] = std::fabs(b.P(i, j, k - 1) - 2.0 * b.P(i, j, k) + b.P(i, j, k + 1)) / pb;
        else
          fp[k] = 0.0;
      }
      fp[0] = 0.0;
      fp[b.kb] = 0.0;
      for (int k = 2; k <= b.ke; k++)
        for (int v = 0; v < 5; v++) diw[k * 5 + v] = b.W(i, j, k, v) - b.W(i, j, k - 1, v);
      for (int v = 0; v < 5; v++) {
        diw[1 * 5 + v] = diw[2 * 5 + v];
        diw[b.kb * 5 + v] = diw[b.ke * 5 + v];
      }
      for (int k = 2; k <= b.ke; k++) {
        double ep = fmax_(fmax_(fmax_(fp[k - 2], fp[k - 1]), fp[k]), fp[k + 1]);
        double out[5], wl[5], wr[5];
        getw(b, i, j, k - 1, wl);
        getw(b, i, j, k, wr);
        face(ep, b.LAM(i, j, k - 1), b.LAM(i, j, k), &diw[(k - 1) * 5], &diw[k * 5], &diw[(k + 1) * 5], wl, wr,
             b.sk, out);
        for (int v = 0; v < 5; v++) dfsz[v * N + b.I(i, j, k)] = out[v];
      }
    }
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 2; k <= b.kl; k++)
    for (int j = 2; j <= b.jl; j++)
      for (int i = 2; i <= b.il; i++)
        for (int v = 0; v < 5; v++)
          b.FW(i, j, k, v) = b.FW(i, j, k, v) + (dfsz[v * N + b.I(i, j, k)] - dfsz[v * N + b.I(i, j, k + 1)]);
  // cut-cell walls, dflux.f90:253
  for (size_t m = 0; m < b.z.size(); m++) dfluxb_rec(c, b, istage, b.z[m], dfsx, dfsy, dfsz);
  // restore the energy, dflux.f90:257-263
  for (size_t q = 0; q < N; q++) b.w[4 * N + q] = we[q];
  return MGE_OK;
}

/* ------------------------------------------------------------------ psmoo.f90:97-242 */
void psmoo_old(mgeo_ctx* c, OBlock& b) {
  const double smoo = c->prm.smoo;
  if (smoo <= 0.0) return;
  const int ilm = b.nx, jlm = b.ny, klm = b.nz, il = b.il, jl = b.jl, kl = b.kl;
  std::vector<double> ex1(il + 1), ex2(il + 1), ey1(jl + 1), ey2(jl + 1), ez1(kl + 1), ez2(kl + 1);
  const double aa = 1.0 + 2.0 * smoo, bb = -smoo;
  auto pivots = [&](std::vector<double>& e1, std::vector<double>& e2, int lm, int l) {
    e1[2] = aa;
    e2[2] = bb / aa;
    for (int q = 3; q <= lm; q++) {
      e1[q] = aa - bb * e2[q - 1];
      e2[q] = bb / e1[q];
    }
    e1[l] = aa - bb * e2[lm];
  };
  pivots(ex1, ex2, ilm, il);
  pivots(ey1, ey2, jlm, jl);
  pivots(ez1, ez2, klm, kl);
  const size_t N = b.N;
  for (int n = 0; n < 5; n++) {
    double* d = &b.dw[n * N];
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int k = 2; k <= kl; k++) {
      for (int j = 2; j <= jl; j++) {  // i-direction, psmoo.f90:173-188
        if (b.BL(2, j, k) != 0) d[b.I(2, j, k)] = d[b.I(2, j, k)] / ex1[2];
        for (int i = 3; i <= il; i++)
          if (b.BL(i, j, k) != 0) d[b.I(i, j, k)] = (d[b.I(i, j, k)] - bb * d[b.I(i - 1, j, k)]) / ex1[i];
        for (int i = 2; i <= ilm; i++) {
          int ir = il + 1 - i;
          if (b.BL(ir, j, k) != 0) d[b.I(ir, j, k)] = d[b.I(ir, j, k)] - ex2[ir] * d[b.I(ir + 1, j, k)];
        }
      }
      for (int i = 2; i <= il; i++) {  // j-direction, psmoo.f90:191-206
        if (b.BL(i, 2, k) != 0) d[b.I(i, 2, k)] = d[b.I(i, 2, k)] / ey1[2];
        for (int j = 3; j <= jl; j++)
          if (b.BL(i, j, k) != 0) d[b.I(i, j, k)] = (d[b.I(i, j, k)] - bb * d[b.I(i, j - 1, k)]) / ey1[j];
        for (int j = 2; j <= jlm; j++) {
          int jr = jl + 1 - j;
          if (b.BL(i, jr, k) != 0) d[b.I(i, jr, k)] = d[b.I(i, jr, k)] - ey2[jr] * d[b.I(i, jr + 1, k)];
        }
      }
    }
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int j = 2; j <= jl; j++) {  // k-direction, psmoo.f90:211-237
      for (int i = 2; i <= il; i++)
        if (b.BL(i, j, 2) != 0) d[b.I(i, j, 2)] = d[b.I(i, j, 2)] / ez1[2];
      for (int k = 3; k <= kl; k++)
        for (int i = 2; i <= il; i++)
          if (b.BL(i, j, k) != 0) d[b.I(i, j, k)] = (d[b.I(i, j, k)] - bb * d[b.I(i, j, k - 1)]) / ez1[k];
      for (int k = 2; k <= klm; k++) {
        int kr = kl + 1 - k;
        for (int i = 2; i <= il; i++)
          if (b.BL(i, j, kr) != 0) d[b.I(i, j, kr)] = d[b.I(i, j, kr)] - ez2[kr] * d[b.I(i, j, kr + 1)];
      }
    }
  }
}

/* progon3.f90:41-60: cyclic tridiagonal sweep */
void progon3(const double* a, const double* bq, const double* cq, const double* d, double* x, int n) {
  std::vector<double> w(n + 2), s(n + 2), t(n + 2), u(n + 2), v(n + 2);
  // Fortran 1-based arrays: element q of a Fortran array is a[q-1]
  u[1] = 0.0;
  v[1] = 0.0;
  w[1] = 1.0;
  for (int i = 1; i <= n; i++) {
    int i1 = i + 1;
    double z = 1.0 / (a[i - 1] + cq[i - 1] * v[i]);
    v[i1] = -bq[i - 1] * z;
    u[i1] = (-cq[i - 1] * u[i] + d[i - 1]) * z;
    w[i1] = -cq[i - 1] * w[i] * z;
  }
  s[n] = 1.0;
  t[n] = 0.0;
  for (int i = n - 1; i >= 1; i--) {
    s[i] = v[i + 1] * s[i + 1] + w[i + 1];
    t[i] = v[i + 1] * t[i + 1] + u[i + 1];
  }
  x[n - 1] = (d[n - 1] - bq[n - 1] * t[1] - cq[n - 1] * t[n - 1]) / (a[n - 1] + bq[n - 1] * s[1] + cq[n - 1] * s[n - 1]);
  for (int i = 1; i <= n - 1; i++) x[i - 1] = s[i] * x[n - 1] + t[i];
}

/* psmoo.f90:1-95 (variable coefficients from timestep, progon3 lines) */
void psmoo_var(mgeo_ctx* c, OBlock& b) {
  if (c->prm.smoo <= 0.0) return;
  const size_t N = b.N;
  const int mx = std::max(b.ib, std::max(b.jb, b.kb));
  auto line = [&](int len, auto idx, const std::vector<double>& eps) {
    std::vector<double> aa(mx + 1), bb(mx + 1), cc(mx + 1), d(mx + 1), x(mx + 1);
    for (int q = 2; q <= len; q++) {
      double e = eps[idx(q)];
      aa[q] = 1.0 + 2.0 * e;
      bb[q] = -e;
      cc[q] = -e;
    }
    bb[len] = 0.0;
    cc[2] = 0.0;
    for (int n = 0; n < 5; n++) {
      for (int q = 2; q <= len; q++) d[q] = b.dw[n * N + idx(q)];
      progon3(&aa[2], &bb[2], &cc[2], &d[2], &x[2], len - 1);
      for (int q = 2; q <= len; q++) b.dw[n * N + idx(q)] = x[q];
    }
  };
  for (int k = 2; k <= b.kl; k++)
    for (int j = 2; j <= b.jl; j++) line(b.il, [&](int q) { return b.I(q, j, k); }, b.epsx);
  for (int k = 2; k <= b.kl; k++)
    for (int i = 2; i <= b.il; i++) line(b.jl, [&](int q) { return b.I(i, q, k); }, b.epsy);
  for (int i = 2; i <= b.il; i++)
    for (int j = 2; j <= b.jl; j++) line(b.kl, [&](int q) { return b.I(i, j, q); }, b.epsz);
}

/* ------------------------------------------------------------------ boundary conditions */
/* bc_far.f90:42-284; face = 1..6 */
void bc_far(mgeo_ctx* c, OBlock& b, int face) {
  const mge_params& P = c->prm;
  const double gamma = P.gamma, gm = 1.0 / (gamma - 1.0);
  const double* fn = b.fnv[face - 1];
  int ax = (face - 1) % 3;  // 0 i, 1 j, 2 k
  int phy1, dum1, dum2;
  int lcur = ax == 0 ? b.il : (ax == 1 ? b.jl : b.kl);
  int ecur = lcur + 1, bcur = lcur + 2;
  if (face <= 3) {
    phy1 = 2;
    dum1 = 1;
    dum2 = 0;
  } else {
    phy1 = lcur;
    dum1 = ecur;
    dum2 = bcur;
  }
  const double u0[3] = {P.u0, P.v0, P.w0};
  int na = ax == 0 ? b.jb : b.ib, nb = ax == 2 ? b.jb : b.kb;
  // loop bounds: face 1/4 over (j,k), face 2/5 over (i,k), face 3/6 over (i,j)
  for (int t2 = 0; t2 <= nb; t2++)
    for (int t1 = 0; t1 <= na; t1++) {
      auto at = [&](int q, int& i, int& j, int& k) {
        if (ax == 0) { i = q; j = t1; k = t2; }
        else if (ax == 1) { i = t1; j = q; k = t2; }
        else { i = t1; j = t2; k = q; }
      };
      int i, j, k;
      at(phy1, i, j, k);
      double wp[5];
      getw(b, i, j, k, wp);
      double pph = b.P(i, j, k);
      double vel_norm = (wp[1] * fn[0] + wp[2] * fn[1] + wp[3] * fn[2]) / wp[0];
      double out[5], pout;
      bool set = false;
      double fnn = fn[ax];
      if (vel_norm <= 0.0) {  // inlet
        double rhoe = wp[0];
        double ue = wp[1 + ax] / rhoe;
        double pe = pph;
        double ce = std::sqrt(gamma * pe / rhoe);
        double rpo = ue * fnn + 2.0 * ce / (gamma - 1.0);
        double rmi = u0[ax] * fnn - 2.0 * P.c0 / (gamma - 1.0);
        double vv[3] = {u0[0], u0[1], u0[2]};
        vv[ax] = 0.5 * (rpo + rmi) * fnn;
        double ci = 0.25 * (gamma - 1.0) * (rpo - rmi);
        double si = std::pow(P.rho0, gamma) / P.p0;
        double cc = ci * ci / gamma;
        double rhoi = std::pow(si * cc, gm);
        double prei = rhoi * cc;
        out[0] = rhoi;
        out[1] = rhoi * vv[0];
        out[2] = rhoi * vv[1];
        out[3] = rhoi * vv[2];
        out[4] = prei * gm + 0.5 * rhoi * (vv[0] * vv[0] + vv[1] * vv[1] + vv[2] * vv[2]);
        pout = prei;
        set = true;
      } else if (vel_norm > 0.0) {  // outlet
        double rhoi = wp[0];
        double vv[3] = {wp[1] / rhoi, wp[2] / rhoi, wp[3] / rhoi};
        double prei = pph;
        double si = std::pow(rhoi, gamma) / prei;
        double ci = std::sqrt(gamma * prei / rhoi);
        double rpo = vv[ax] * fnn + 2.0 * ci / (gamma - 1.0);
        double rmi = u0[ax] * fnn - 2.0 * P.c0 / (gamma - 1.0);
        double ve[3] = {vv[0], vv[1], vv[2]};
        ve[ax] = 0.5 * (rpo + rmi) * fnn;
        double ce = 0.25 * (gamma - 1.0) * (rpo - rmi);
        double se = si;
        double cc = ce * ce / gamma;
        double rhoe = std::pow(se * cc, gm);
        double pe = rhoe * cc;
        out[0] = rhoe;
        out[1] = rhoe * ve[0];
        out[2] = rhoe * ve[1];
        out[3] = rhoe * ve[2];
        out[4] = pe * gm + 0.5 * rhoe * (ve[0] * ve[0] + ve[1] * ve[1] + ve[2] * ve[2]);
        pout = pe;
        set = true;
      }
      int i1, j1, k1, i2, j2, k2;
      at(dum1, i1, j1, k1);
      at(dum2, i2, j2, k2);
      if (set) {
        for (int v = 0; v < 5; v++) b.W(i1, j1, k1, v) = out[v];
        b.P(i1, j1, k1) = pout;
      }
      for (int v = 0; v < 5; v++) b.W(i2, j2, k2, v) = b.W(i1, j1, k1, v);
      b.P(i2, j2, k2) = b.P(i1, j1, k1);
    }
}

/* bc_symm.f90:27-82, bc_wall.f90:28-89, bc_periodic.f90:27-91 */
void bc_copy_face(OBlock& b, int face, int kind) {
  int ax = (face - 1) % 3;
  int lcur = ax == 0 ? b.il : (ax == 1 ? b.jl : b.kl);
  int phy1, phy2, dum1, dum2;
  if (kind == -60) {  // periodic
    if (face <= 3) {
      dum1 = 1; dum2 = 0; phy1 = lcur; phy2 = lcur - 1;
    } else {
      phy1 = 2; phy2 = 3; dum1 = lcur + 1; dum2 = lcur + 2;
    }
  } else {
    if (face <= 3) {
      phy1 = 2; phy2 = 3; dum1 = 1; dum2 = 0;
    } else {
      phy1 = lcur; phy2 = lcur - 1; dum1 = lcur + 1; dum2 = lcur + 2;
    }
  }
  int na = ax == 0 ? b.jb : b.ib, nb = ax == 2 ? b.jb : b.kb;
  for (int t2 = 0; t2 <= nb; t2++)
    for (int t1 = 0; t1 <= na; t1++) {
      auto id = [&](int q) {
        if (ax == 0) return b.I(q, t1, t2);
        if (ax == 1) return b.I(t1, q, t2);
        return b.I(t1, t2, q);
      };
      size_t d1 = id(dum1), d2 = id(dum2), p1 = id(phy1), p2 = id(phy2);
      const size_t N = b.N;
      if (kind == -50) {  // symmetry: mirror the face-normal momentum
        for (int v = 0; v < 5; v++) b.w[v * N + d1] = b.w[v * N + p1];
        b.w[(1 + ax) * N + d1] = -b.w[(1 + ax) * N + p1];
        b.p[d1] = b.p[p1];
        for (int v = 0; v < 5; v++) b.w[v * N + d2] = b.w[v * N + p2];
        b.w[(1 + ax) * N + d2] = -b.w[(1 + ax) * N + p2];
        b.p[d2] = b.p[p2];
      } else if (kind == -80) {  // no-slip wall
        b.w[0 * N + d1] = b.w[0 * N + p1];
        b.w[4 * N + d1] = b.w[4 * N + p1];
        for (int v = 1; v < 4; v++) b.w[v * N + d1] = -b.w[v * N + p1];
        b.w[0 * N + d2] = b.w[0 * N + p2];
        b.w[4 * N + d2] = b.w[4 * N + p2];
        for (int v = 1; v < 4; v++) b.w[v * N + d2] = -b.w[v * N + p2];
        b.p[d1] = b.p[p1];
        b.p[d2] = b.p[p1];
      } else {  // periodic
        for (int v = 0; v < 5; v++) b.w[v * N + d2] = b.w[v * N + p2];
        for (int v = 0; v < 5; v++) b.w[v * N + d1] = b.w[v * N + p1];
        b.p[d2] = b.p[p2];
        b.p[d1] = b.p[p1];
      }
    }
}

/* bc_corner.f90:23-157 */
void bc_corner(mgeo_ctx* c, OBlock& b) {
  const mge_params& P = c->prm;
  const int il = b.il, jl = b.jl, kl = b.kl, ie = b.ie, je = b.je, ke = b.ke;
  auto set3 = [&](int i, int j, int k, int ia, int ja, int ka, int ib_, int jb_, int kb_, int ic, int jc, int kc) {
    for (int v = 0; v < 5; v++) b.W(i, j, k, v) = b.W(ia, ja, ka, v) + b.W(ib_, jb_, kb_, v) - b.W(ic, jc, kc, v);
    depvars_cell(P, b, i, j, k);
  };
  for (int k = 2; k <= kl; k++) {
    set3(1, 1, k, 2, 1, k, 1, 2, k, 2, 2, k);
    set3(ie, 1, k, il, 1, k, ie, 2, k, il, 2, k);
    set3(1, je, k, 2, je, k, 1, jl, k, 2, jl, k);
    set3(ie, je, k, il, je, k, ie, jl, k, il, jl, k);
  }
  for (int j = 2; j <= jl; j++) {
    set3(1, j, 1, 2, j, 1, 1, j, 2, 2, j, 2);
    set3(ie, j, 1, il, j, 1, ie, j, 2, il, j, 2);
    set3(1, j, ke, 2, j, ke, 1, j, kl, 2, j, kl);
    set3(ie, j, ke, il, j, ke, ie, j, kl, il, j, kl);
  }
  for (int i = 0; i <= b.ib; i++) {
    set3(i, 1, 1, i, 1, 2, i, 2, 1, i, 2, 2);
    set3(i, 1, ke, i, 2, ke, i, 1, kl, i, 2, kl);
    set3(i, je, 1, i, je, 1, i, jl, 2, i, jl, 2);  // bc_corner.f90:120 as written
    set3(i, je, ke, i, jl, ke, i, je, kl, i, jl, kl);
  }
  auto c8 = [&](int i, int j, int k, int ia, int ja, int ka, int ib_, int jb_, int kb_, int ic, int jc, int kc, int id,
                int jd, int kd) {
    for (int v = 0; v < 5; v++)
      b.W(i, j, k, v) =
          (b.W(ia, ja, ka, v) + b.W(ib_, jb_, kb_, v) + b.W(ic, jc, kc, v)) * 2.0 / 3.0 - b.W(id, jd, kd, v);
  };
  c8(1, 1, 1, 2, 1, 1, 1, 2, 1, 1, 1, 2, 2, 2, 2);
  c8(1, 1, ke, 2, 1, ke, 1, 2, ke, 1, 1, kl, 2, 2, kl);
  c8(1, je, 1, 2, je, 1, 1, jl, 1, 1, je, 2, 2, jl, 2);
  c8(ie, 1, 1, il, 1, 1, ie, 2, 1, ie, 1, 2, il, 2, 2);
  c8(ie, 1, ke, il, 1, ke, ie, 2, ke, ie, 1, kl, il, 2, kl);
  c8(ie, je, 1, il, je, 1, ie, jl, 1, ie, je, 2, il, jl, 2);
  c8(1, je, ke, 2, je, ke, 1, jl, ke, 1, je, kl, 2, jl, kl);
  c8(ie, je, ke, il, je, ke, ie, jl, ke, ie, je, kl, il, jl, kl);
  depvars_cell(P, b, 1, 1, 1);
  depvars_cell(P, b, 1, 1, ke);
  depvars_cell(P, b, 1, je, 1);
  depvars_cell(P, b, ie, 1, 1);
  depvars_cell(P, b, ie, 1, ke);
  depvars_cell(P, b, ie, je, 1);
  depvars_cell(P, b, 1, je, ke);
  depvars_cell(P, b, ie, je, ke);
}

/* bcond.f90:16-42 */
int bcond(mgeo_ctx* c, OBlock& b) {
  for (int f = 1; f <= 6; f++) {
    int t = b.bctype[f - 1];
    if (t == 0) continue;
    if (t == -20) bc_far(c, b, f);
    else if (t == -50) bc_copy_face(b, f, -50);
    else if (t == -60) {
      bc_copy_face(b, f, -60);
      if (f <= 3 && b.bctype[f + 2] != -60)
        return fail(c, MGE_EBADCFG, "periodic boundary must appear in pairs (bcond.f90:26-31)");
    } else if (t == -80) bc_copy_face(b, f, -80);
    // other codes: the reference prints and continues
  }
  bc_corner(c, b);
  return MGE_OK;
}

/* bc_cutcell.f90:40-268.  The normal and the wall velocity are the record's:
   the descriptor's nvec and qb (approxbc off, qb 0 for a fixed wall), or
   norv and vel/vel_fs after mgeo_move_surface (approxbc on, :47-50) */
int bc_cutcell(mgeo_ctx* c, OBlock& b) {
  const mge_params& P = c->prm;
  for (size_t m = 0; m < b.z.size(); m++) {
    ORec& t = b.z[m];
    int ncl = t.npoint;
    double nvec[3] = {t.nvec[0], t.nvec[1], t.nvec[2]};
    double qb[3] = {t.qb[0], t.qb[1], t.qb[2]};
    double nn = std::sqrt(nvec[0] * nvec[0] + nvec[1] * nvec[1] + nvec[2] * nvec[2]);
    for (int q = 0; q < 3; q++) nvec[q] = nvec[q] / nn;
    double psol = 0.0, wsol[5] = {0, 0, 0, 0, 0};
    if (ncl == 0) {  // bc_cutcell.f90:65-70: warn, zero this record, leave the routine
      t.psol = psol;
      for (int v = 0; v < 5; v++) t.wsol[v] = wsol[v];
      return MGE_OK;
    }
    double var_refl[5] = {0, 0, 0, 0, 0};
    for (int v = 0; v < 5; v++)
      for (int q = 0; q < ncl; q++) var_refl[v] = var_refl[v] + t.coef[q] * b.W(t.ijk[q][0], t.ijk[q][1], t.ijk[q][2], v);
    double p_refl = 0.0;
    for (int q = 0; q < ncl; q++) p_refl = p_refl + t.coef[q] * b.P(t.ijk[q][0], t.ijk[q][1], t.ijk[q][2]);
    if (P.eqntype == MGE_EQN_EULER) {
      psol = p_refl;
      for (int v = 0; v < 5; v++) wsol[v] = var_refl[v];
      double qn = 2.0 * (nvec[0] * (wsol[1] - wsol[0] * qb[0]) + nvec[1] * (wsol[2] - wsol[0] * qb[1]) +
                         nvec[2] * (wsol[3] - wsol[0] * qb[2]));
      for (int q = 0; q < 3; q++) wsol[1 + q] = wsol[1 + q] - qn * nvec[q];
      wsol[4] = psol / (P.gamma - 1.0) + 0.5 * (wsol[1] * wsol[1] + wsol[2] * wsol[2] + wsol[3] * wsol[3]) / wsol[0];
      for (int v = 0; v < 5; v++)
        if (wsol[v] != wsol[v]) return fail(c, MGE_ENAN, "bc_cutcell: wsol is NaN (bc_cutcell.f90:147-156)");
    } else {
      psol = p_refl;
      for (int v = 0; v < 5; v++) wsol[v] = var_refl[v];
      for (int q = 0; q < 3; q++) wsol[1 + q] = 2.0 * qb[q] * var_refl[0] - var_refl[1 + q];  // option B, :185
      wsol[4] = psol / (P.gamma - 1.0) + 0.5 * (wsol[1] * wsol[1] + wsol[2] * wsol[2] + wsol[3] * wsol[3]) / wsol[0];
    }
    t.psol = psol;
    for (int v = 0; v < 5; v++) t.wsol[v] = wsol[v];
  }
  return MGE_OK;
}

/* ------------------------------------------------------------------ Roe and viscous fluxes
 * The reference selects these with distype 'r1'/'r2' and eqntype 'n'
 * (euler.f90:137-210) but their sources (roepak, viscpak) are not part of
 * its tree, so this build defines them from the published methods:
 *  - Roe's approximate Riemann solver (P. L. Roe, J. Comput. Phys. 43, 1981)
 *    with Harten's entropy fix (A. Harten, J. Comput. Phys. 49, 1983),
 *    split like the JST scheme: the central part 0.5*(F(U_L)+F(U_R)).s goes
 *    to dw, the upwind part 0.5*cdis(m)*|s|*|A|(U_R-U_L) to fw;
 *  - 'r2': MUSCL reconstruction of (rho,u,v,w,p) with the van Albada
 *    limiter, first order on any face whose 4-cell stencil touches a blanked
 *    cell;
 *  - laminar viscous flux with face gradients from central differences (the
 *    normal one across the face, tangential ones averaged over the two
 *    cells), Stokes stresses and Fourier heat flux, scaled by cdis(m) and
 *    added to fw before the dissipation (euler.f90:157-181);
 *  - cut-cell walls: the wall face of each record is replaced, for the Roe
 *    dissipation by the flux to the ghost state (wsol,psol), for the viscous
 *    flux by the no-slip adiabatic wall flux (normal gradients only, zero
 *    heat flux).
 */
struct Prim {
  double r, u[3], p;
};
inline Prim to_prim(const double* w, double p) {
  Prim q;
  q.r = w[0];
  for (int a = 0; a < 3; a++) q.u[a] = w[1 + a] / w[0];
  q.p = p;
  return q;
}
inline void to_cons(double gamma, const Prim& q, double* w) {
  w[0] = q.r;
  for (int a = 0; a < 3; a++) w[1 + a] = q.r * q.u[a];
  w[4] = q.p / (gamma - 1.0) + 0.5 * q.r * (q.u[0] * q.u[0] + q.u[1] * q.u[1] + q.u[2] * q.u[2]);
}
// van Albada limited slope of two one-sided differences
// van Albada's limited slope (van Albada, van Leer & Roberts 1982) in its
// smooth form with e2 = eps^2; no cut-off at a*b <= 0, which with e2 > 0
// would make the slope jump by up to b/3 when a changes sign
inline double van_albada(double a, double b, double e2) {
  return ((b * b + e2) * a + (a * a + e2) * b) / (a * a + b * b + 2.0 * e2);
}
// upwind dissipation 0.5*|s|*|A_roe|(U_R-U_L) along axis d with Harten's fix
void roe_dissipation(const mge_params& P, int d, double S, const double* wl, double pl, const double* wr, double pr,
                     double* out) {
  const double g = P.gamma;
  double ul[3], ur[3];
  for (int a = 0; a < 3; a++) {
    ul[a] = wl[1 + a] / wl[0];
    ur[a] = wr[1 + a] / wr[0];
  }
  double hl = (wl[4] + pl) / wl[0], hr = (wr[4] + pr) / wr[0];
  double rt = std::sqrt(wr[0] / wl[0]);
  double rh = rt * wl[0];
  double uh[3];
  for (int a = 0; a < 3; a++) uh[a] = (ul[a] + rt * ur[a]) / (1.0 + rt);
  double hh = (hl + rt * hr) / (1.0 + rt);
  double q2 = uh[0] * uh[0] + uh[1] * uh[1] + uh[2] * uh[2];
  double c2 = (g - 1.0) * (hh - 0.5 * q2);
  double ch = std::sqrt(fmax_(c2, 1e-300));
  double un = uh[d];
  double dr = wr[0] - wl[0], dp = pr - pl, dun = ur[d] - ul[d];
  double du[3] = {ur[0] - ul[0], ur[1] - ul[1], ur[2] - ul[2]};
  double delta = P.epsentr * (std::fabs(un) + ch);
  auto fix = [&](double lam) {
    double a = std::fabs(lam);
    return (a < delta && delta > 0.0) ? (lam * lam + delta * delta) / (2.0 * delta) : a;
  };
  double l1 = fix(un - ch), l2 = fix(un), l5 = fix(un + ch);
  double a1 = (dp - rh * ch * dun) / (2.0 * c2);
  double a2 = dr - dp / c2;
  double a5 = (dp + rh * ch * dun) / (2.0 * c2);
  double sh[3];
  for (int a = 0; a < 3; a++) sh[a] = rh * (du[a] - (a == d ? dun : 0.0));
  double k1[5], k5[5];
  k1[0] = 1.0;
  k5[0] = 1.0;
  for (int a = 0; a < 3; a++) {
    k1[1 + a] = uh[a] - (a == d ? ch : 0.0);
    k5[1 + a] = uh[a] + (a == d ? ch : 0.0);
  }
  k1[4] = hh - ch * un;
  k5[4] = hh + ch * un;
  double res[5];
  res[0] = l1 * a1 * k1[0] + l2 * a2 + l5 * a5 * k5[0];
  for (int a = 0; a < 3; a++) res[1 + a] = l1 * a1 * k1[1 + a] + l2 * (a2 * uh[a] + sh[a]) + l5 * a5 * k5[1 + a];
  res[4] = l1 * a1 * k1[4] + l2 * (a2 * 0.5 * q2 + (uh[0] * sh[0] + uh[1] * sh[1] + uh[2] * sh[2])) + l5 * a5 * k5[4];
  for (int v = 0; v < 5; v++) out[v] = 0.5 * S * res[v];
}

// left/right states of face q (between q-1 and q) along axis d at (i,j,k) = cell q
void face_states(mgeo_ctx* c, OBlock& b, int d, int i, int j, int k, int order, double* wl, double* pl, double* wr,
                 double* pr) {
  const mge_params& P = c->prm;
  int e[3] = {0, 0, 0};
  e[d] = 1;
  auto W = [&](int o, int v) { return b.W(i + o * e[0], j + o * e[1], k + o * e[2], v); };
  auto PP = [&](int o) { return b.P(i + o * e[0], j + o * e[1], k + o * e[2]); };
  auto BLK = [&](int o) { return b.BL(i + o * e[0], j + o * e[1], k + o * e[2]); };
  for (int v = 0; v < 5; v++) {
    wl[v] = W(-1, v);
    wr[v] = W(0, v);
  }
  *pl = PP(-1);
  *pr = PP(0);
  if (order < 2) return;
  const int q = d == 0 ? i : (d == 1 ? j : k);
  const int lq = d == 0 ? b.il : (d == 1 ? b.jl : b.kl);
  if (q - 2 < 0 || q + 1 > lq + 2) return;
  if (BLK(-2) == 0 || BLK(-1) == 0 || BLK(0) == 0 || BLK(1) == 0) return;  // first order next to the body
  double wt[4][5], pt[4];
  for (int o = -2; o <= 1; o++) {
    for (int v = 0; v < 5; v++) wt[o + 2][v] = W(o, v);
    pt[o + 2] = PP(o);
  }
  Prim m2 = to_prim(wt[0], pt[0]), m1 = to_prim(wt[1], pt[1]), z0 = to_prim(wt[2], pt[2]), p1 = to_prim(wt[3], pt[3]);
  const double u0n = std::sqrt(P.u0 * P.u0 + P.v0 * P.v0 + P.w0 * P.w0);
  const double ref[5] = {P.rho0, u0n, u0n, u0n, P.p0};
  auto lim = [&](double a, double bb, int kq) {
    double e2 = 1e-6 * ref[kq] * ref[kq] / (P.limfac > 0.0 ? P.limfac : 1.0);
    return van_albada(a, bb, e2);
  };
  auto comp = [&](const Prim& x, int kq) { return kq == 0 ? x.r : (kq == 4 ? x.p : x.u[kq - 1]); };
  Prim L = m1, R = z0;
  for (int kq = 0; kq < 5; kq++) {
    double dm = comp(m1, kq) - comp(m2, kq), d0 = comp(z0, kq) - comp(m1, kq), dp = comp(p1, kq) - comp(z0, kq);
    double sl = 0.5 * lim(dm, d0, kq), sr = 0.5 * lim(d0, dp, kq);
    if (kq == 0) { L.r = m1.r + sl; R.r = z0.r - sr; }
    else if (kq == 4) { L.p = m1.p + sl; R.p = z0.p - sr; }
    else { L.u[kq - 1] = m1.u[kq - 1] + sl; R.u[kq - 1] = z0.u[kq - 1] - sr; }
  }
  if (L.r <= 0.0 || R.r <= 0.0 || L.p <= 0.0 || R.p <= 0.0) return;  // keep first order where the reconstruction fails
  to_cons(P.gamma, L, wl);
  to_cons(P.gamma, R, wr);
  *pl = L.p;
  *pr = R.p;
}

// Roe scheme: central part into dw (with efluxb at walls), upwind part into fw
int roe_fluxes(mgeo_ctx* c, OBlock& b, int istage) {
  const mge_params& P = c->prm;
  const int order = P.distype == MGE_DIS_ROE2 ? 2 : 1;
  const size_t N = b.N;
  const double cd = P.cdis[istage - 1];
  int rc;
  if (order == 1) {
    rc = eflux(c, b);  // the central part of Roe's flux with cell states is eflux's
    if (rc) return rc;
  } else {
    std::vector<double> E(15 * N, 0.0);
    const double* sv[3] = {b.si, b.sj, b.sk};
    for (int d = 0; d < 3; d++) {
      int lo[3] = {2, 2, 2}, hi[3] = {b.il, b.jl, b.kl};
      hi[d] += 1;
#pragma omp parallel for num_threads(g_threads) schedule(static)
      for (int k = lo[2]; k <= hi[2]; k++)
        for (int j = lo[1]; j <= hi[1]; j++)
          for (int i = lo[0]; i <= hi[0]; i++) {
            double wl[5], wr[5], pl, pr, f1[5], f2[5];
            face_states(c, b, d, i, j, k, 2, wl, &pl, wr, &pr);
            ceflux(wr, pr, sv[d], f1);
            ceflux(wl, pl, sv[d], f2);
            for (int v = 0; v < 5; v++) E[(d * 5 + v) * N + b.I(i, j, k)] = 0.5 * (f1[v] + f2[v]);
          }
    }
    const size_t st[3] = {1, b.Pi, b.Pi * b.Pj};
    for (int k = 2; k <= b.kl; k++)
      for (int j = 2; j <= b.jl; j++)
        for (int i = 2; i <= b.il; i++) {
          size_t q = b.I(i, j, k);
          for (int v = 0; v < 5; v++) {
            double a = E[(0 * 5 + v) * N + q] - E[(0 * 5 + v) * N + q + st[0]];
            a = a + E[(1 * 5 + v) * N + q] - E[(1 * 5 + v) * N + q + st[1]];
            a = a + E[(2 * 5 + v) * N + q] - E[(2 * 5 + v) * N + q + st[2]];
            b.dw[v * N + q] = a;
          }
        }
    // walls: efluxb's replacement of the wall face (efluxb.f90:30-114)
    for (size_t m = 0; m < b.z.size(); m++) {
      ORec& t = b.z[m];
      int D = t.zz - 1, i = t.ccid[0], j = t.ccid[1], k = t.ccid[2];
      if (std::fabs(b.W(i, j, k, 0)) < 1.0e-8) return fail(c, MGE_EZERORHO, "zero density at a cut cell");
      const double* sc = sv[D];
      double wc[5], wn[5], f1[5], f2[5], f3[5];
      getw(b, i, j, k, wc);
      ceflux(wc, b.P(i, j, k), sc, f1);
      ceflux(t.wsol, t.psol, sc, f2);
      int di = D == 0, dj = D == 1, dk = D == 2;
      size_t q = b.I(i, j, k), qn = b.I(i + di, j + dj, k + dk);
      for (int v = 0; v < 5; v++) b.dw[v * N + q] = b.dw[v * N + q] - (E[(D * 5 + v) * N + q] - E[(D * 5 + v) * N + qn]);
      bool plus = t.faceid >= 4;
      int s = plus ? -1 : 1;
      getw(b, i + s * di, j + s * dj, k + s * dk, wn);
      ceflux(wn, b.P(i + s * di, j + s * dj, k + s * dk), sc, f3);
      for (int v = 0; v < 5; v++) {
        double fs = 0.5 * (f1[v] + f2[v]), fa = 0.5 * (f1[v] + f3[v]);
        b.dw[v * N + q] = b.dw[v * N + q] + (plus ? fa : fs) - (plus ? fs : fa);
      }
    }
  }
  if (cd <= 0.0) return MGE_OK;
  // upwind dissipation faces
  std::vector<double> D(15 * N, 0.0);
  const double Sd[3] = {std::fabs(b.si[0]), std::fabs(b.sj[1]), std::fabs(b.sk[2])};
  for (int d = 0; d < 3; d++) {
    int lo[3] = {2, 2, 2}, hi[3] = {b.il, b.jl, b.kl};
    hi[d] += 1;
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int k = lo[2]; k <= hi[2]; k++)
      for (int j = lo[1]; j <= hi[1]; j++)
        for (int i = lo[0]; i <= hi[0]; i++) {
          double wl[5], wr[5], pl, pr, o[5];
          face_states(c, b, d, i, j, k, order, wl, &pl, wr, &pr);
          roe_dissipation(P, d, Sd[d], wl, pl, wr, pr, o);
          for (int v = 0; v < 5; v++) D[(d * 5 + v) * N + b.I(i, j, k)] = cd * o[v];
        }
  }
  const size_t st[3] = {1, b.Pi, b.Pi * b.Pj};
  for (int d = 0; d < 3; d++)
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int k = 2; k <= b.kl; k++)
      for (int j = 2; j <= b.jl; j++)
        for (int i = 2; i <= b.il; i++) {
          size_t q = b.I(i, j, k);
          for (int v = 0; v < 5; v++)
            b.fw[v * N + q] = b.fw[v * N + q] + (D[(d * 5 + v) * N + q] - D[(d * 5 + v) * N + q + st[d]]);
        }
  // walls: the wall face's upwind flux taken to the ghost state
  for (size_t m = 0; m < b.z.size(); m++) {
    ORec& t = b.z[m];
    int d = t.zz - 1, i = t.ccid[0], j = t.ccid[1], k = t.ccid[2];
    size_t q = b.I(i, j, k);
    bool plus = t.faceid >= 4;
    double wc[5], o[5], X[5], Z[5];
    getw(b, i, j, k, wc);
    if (plus) {
      roe_dissipation(P, d, Sd[d], wc, b.P(i, j, k), t.wsol, t.psol, o);
      for (int v = 0; v < 5; v++) {
        X[v] = -D[(d * 5 + v) * N + q + st[d]];
        Z[v] = -(cd * o[v]);
      }
    } else {
      roe_dissipation(P, d, Sd[d], t.wsol, t.psol, wc, b.P(i, j, k), o);
      for (int v = 0; v < 5; v++) {
        X[v] = D[(d * 5 + v) * N + q];
        Z[v] = cd * o[v];
      }
    }
    for (int v = 0; v < 5; v++) {
      b.fw[v * N + q] = b.fw[v * N + q] - X[v];
      b.fw[v * N + q] = b.fw[v * N + q] + Z[v];
    }
  }
  return MGE_OK;
}

// laminar viscous flux through the face of cell q along d (euler.f90:137-181, this build's definition)
void visc_face(const mge_params& P, OBlock& b, const std::vector<double>& vel, const std::vector<double>& tem, int d,
               int i, int j, int k, double S, double* out) {
  const size_t N = b.N;
  int e[3] = {0, 0, 0};
  e[d] = 1;
  size_t qR = b.I(i, j, k), qL = b.I(i - e[0], j - e[1], k - e[2]);
  double g[4][3];  // d(u,v,w,T)/dx_t
  for (int a = 0; a < 4; a++) {
    const double* f = a < 3 ? &vel[a * N] : tem.data();
    for (int t = 0; t < 3; t++) {
      if (t == d) {
        g[a][t] = (f[qR] - f[qL]) / b.h[d];
      } else {
        int o[3] = {0, 0, 0};
        o[t] = 1;
        size_t rp = b.I(i + o[0], j + o[1], k + o[2]), rm = b.I(i - o[0], j - o[1], k - o[2]);
        size_t lp = b.I(i - e[0] + o[0], j - e[1] + o[1], k - e[2] + o[2]);
        size_t lm = b.I(i - e[0] - o[0], j - e[1] - o[1], k - e[2] - o[2]);
        g[a][t] = ((f[rp] - f[rm]) + (f[lp] - f[lm])) / (4.0 * b.h[t]);
      }
    }
  }
  const double mu = P.viscl;
  const double kt = mu * P.gamma * P.gas_const / ((P.gamma - 1.0) * P.prlmean);
  double div = g[0][0] + g[1][1] + g[2][2];
  double tau[3];
  for (int a = 0; a < 3; a++) tau[a] = mu * (g[a][d] + g[d][a]) - (a == d ? (2.0 / 3.0) * mu * div : 0.0);
  double uf[3];
  for (int a = 0; a < 3; a++) uf[a] = 0.5 * (vel[a * N + qL] + vel[a * N + qR]);
  out[0] = 0.0;
  for (int a = 0; a < 3; a++) out[1 + a] = S * tau[a];
  out[4] = S * ((uf[0] * tau[0] + uf[1] * tau[1] + uf[2] * tau[2]) + kt * g[3][d]);
}

// no-slip adiabatic wall face of a record: normal gradients to the mirror state only
void visc_wall(const mge_params& P, OBlock& b, const ORec& t, double S, double* out) {
  int d = t.zz - 1;
  bool plus = t.faceid >= 4;
  double u[3], ug[3], qb[3] = {t.qb[0], t.qb[1], t.qb[2]};
  for (int a = 0; a < 3; a++) {
    u[a] = b.W(t.ccid[0], t.ccid[1], t.ccid[2], 1 + a) / b.W(t.ccid[0], t.ccid[1], t.ccid[2], 0);
    ug[a] = 2.0 * qb[a] - u[a];
  }
  double gn[3];
  for (int a = 0; a < 3; a++) gn[a] = plus ? (ug[a] - u[a]) / b.h[d] : (u[a] - ug[a]) / b.h[d];
  const double mu = P.viscl;
  double tau[3];
  for (int a = 0; a < 3; a++) tau[a] = (a == d) ? (4.0 / 3.0) * mu * gn[a] : mu * gn[a];
  out[0] = 0.0;
  for (int a = 0; a < 3; a++) out[1 + a] = S * tau[a];
  out[4] = S * (qb[0] * tau[0] + qb[1] * tau[1] + qb[2] * tau[2]);
}

int vflux_all(mgeo_ctx* c, OBlock& b, int istage) {
  const mge_params& P = c->prm;
  const double cd = P.cdis[istage - 1];
  const size_t N = b.N;
  std::vector<double> vel(3 * N), tem(N);
  for (size_t q = 0; q < N; q++) {  // euler.f90:140-154
    double w0 = b.w[q];
    for (int a = 0; a < 3; a++) vel[a * N + q] = b.w[(1 + a) * N + q] / w0;
    tem[q] = b.p[q] / (w0 * P.gas_const);
    if (b.blank[q] == 0) {
      for (int a = 0; a < 3; a++) vel[a * N + q] = 0.0;
      tem[q] = 0.0;
    }
  }
  const double Sd[3] = {std::fabs(b.si[0]), std::fabs(b.sj[1]), std::fabs(b.sk[2])};
  const size_t st[3] = {1, b.Pi, b.Pi * b.Pj};
  std::vector<double> V(15 * N, 0.0);
  for (int d = 0; d < 3; d++) {
    int hi[3] = {b.il, b.jl, b.kl};
    hi[d] += 1;
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int k = 2; k <= hi[2]; k++)
      for (int j = 2; j <= hi[1]; j++)
        for (int i = 2; i <= hi[0]; i++) {
          double o[5];
          visc_face(P, b, vel, tem, d, i, j, k, Sd[d], o);
          for (int v = 0; v < 5; v++) V[(d * 5 + v) * N + b.I(i, j, k)] = cd * o[v];
        }
  }
  for (int d = 0; d < 3; d++)
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int k = 2; k <= b.kl; k++)
      for (int j = 2; j <= b.jl; j++)
        for (int i = 2; i <= b.il; i++) {
          size_t q = b.I(i, j, k);
          for (int v = 0; v < 5; v++)
            b.fw[v * N + q] = b.fw[v * N + q] + (V[(d * 5 + v) * N + q] - V[(d * 5 + v) * N + q + st[d]]);
        }
  for (size_t m = 0; m < b.z.size(); m++) {  // walls, record order
    const ORec& t = b.z[m];
    int d = t.zz - 1;
    size_t q = b.I(t.ccid[0], t.ccid[1], t.ccid[2]);
    bool plus = t.faceid >= 4;
    double o[5], X[5], Z[5];
    visc_wall(P, b, t, Sd[d], o);
    for (int v = 0; v < 5; v++) {
      if (plus) {
        X[v] = -V[(d * 5 + v) * N + q + st[d]];
        Z[v] = -(cd * o[v]);
      } else {
        X[v] = V[(d * 5 + v) * N + q];
        Z[v] = cd * o[v];
      }
      b.fw[v * N + q] = b.fw[v * N + q] - X[v];
      b.fw[v * N + q] = b.fw[v * N + q] + Z[v];
    }
  }
  return MGE_OK;
}

/* ------------------------------------------------------------------ euler.f90:1-462 */
int euler(mgeo_ctx* c, OBlock& b, int itime, int ncyc, int mgl, int mlvl, bool lres, bool lfir, int nstage_limit) {
  const mge_params& P = c->prm;
  const bool unsteady = P.execmode == 1;
  const size_t N = b.N;
  const double fcoll = 1.0;
  if (lfir) b.ws = b.w;  // euler.f90:75-77
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int k = 2; k <= b.kl; k++)
    for (int j = 2; j <= b.jl; j++)
      for (int i = 2; i <= b.il; i++)
        for (int v = 0; v < 5; v++) b.wn[v * N + b.I(i, j, k)] = b.W(i, j, k, v);
  std::fill(b.dw.begin(), b.dw.end(), 0.0);
  std::fill(b.fw.begin(), b.fw.end(), 0.0);
  const int mstage = std::min(P.mstage, nstage_limit > 0 ? nstage_limit : P.mstage);
  for (int m = 1; m <= mstage; m++) {
    double fn = P.cstp[m - 1] * P.cfl;
    if (m > 1) {
      double f = 1.0 - P.cdis[m - 1];
#pragma omp parallel for num_threads(g_threads) schedule(static)
      for (int k = 2; k <= b.kl; k++)
        for (int j = 2; j <= b.jl; j++)
          for (int i = 2; i <= b.il; i++)
            for (int v = 0; v < 5; v++) b.FW(i, j, k, v) = b.FW(i, j, k, v) * f;
    }
    int rc;
    if (P.eqntype == MGE_EQN_NS && P.cdis[m - 1] > 0.0) {  // euler.f90:137-182
      rc = vflux_all(c, b, m);
      if (rc) return rc;
    }
    if (P.distype == MGE_DIS_CENTRAL) {
      if (P.cdis[m - 1] > 0.0) {
        rc = dflux(c, b, m);
        if (rc) return rc;
      }
      rc = eflux(c, b);
      if (rc) return rc;
    } else if (P.distype == MGE_DIS_ROE1 || P.distype == MGE_DIS_ROE2) {
      rc = roe_fluxes(c, b, m);
      if (rc) return rc;
    } else {
      return fail(c, MGE_EBADCFG, "distype should be c/r1/r2 (euler.f90:212-214)");
    }
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int k = 2; k <= b.kl; k++)
      for (int j = 2; j <= b.jl; j++)
        for (int i = 2; i <= b.il; i++)
          for (int v = 0; v < 5; v++) b.DW(i, j, k, v) = b.DW(i, j, k, v) + b.FW(i, j, k, v);
    if (unsteady && itime >= 1) {  // euler.f90:249-275: BDF2, or the first step's (halved) BDF1
      const double f = 0.5 * b.vol / P.dtstep;
#pragma omp parallel for num_threads(g_threads) schedule(static)
      for (int k = 2; k <= b.kl; k++)
        for (int j = 2; j <= b.jl; j++)
          for (int i = 2; i <= b.il; i++) {
            const size_t q = b.I(i, j, k);
            for (int v = 0; v < 5; v++) {
              const size_t x = v * N + q;
              if (itime > 1)
                b.dw[x] = b.dw[x] + f * (3.0 * b.w[x] - 4.0 * b.w1[x] + b.w2[x]);
              else
                b.dw[x] = b.dw[x] + f * (b.w[x] - b.w1[x]);
            }
          }
    }
    if (mgl < mlvl) {  // euler.f90:294-318
      const bool first = lfir && m == 1;
#pragma omp parallel for num_threads(g_threads) schedule(static)
      for (int k = 2; k <= b.kl; k++)
        for (int j = 2; j <= b.jl; j++)
          for (int i = 2; i <= b.il; i++) {
            size_t q = b.I(i, j, k);
            for (int v = 0; v < 5; v++) {
              if (first) {
                b.qf[v * N + q] = 0.0;
                if (b.marker[q] == 1) b.qf[v * N + q] = fcoll * b.wr[v * N + q] - b.dw[v * N + q];
              }
              b.dw[v * N + q] = b.dw[v * N + q] + b.qf[v * N + q];
            }
          }
      if (unsteady) {  // euler.f90:320-331
#pragma omp parallel for num_threads(g_threads) schedule(static)
        for (int k = 2; k <= b.kl; k++)
          for (int j = 2; j <= b.jl; j++)
            for (int i = 2; i <= b.il; i++) {
              double de = fn * b.vdtim[b.I(i, j, k)];
              if (P.vt == 1) de = fn * b.dtim;
              const double lam = 1.0 + de * 3.0 / 2.0 / P.dtstep;
              for (int v = 0; v < 5; v++) b.DW(i, j, k, v) = b.DW(i, j, k, v) / lam;
            }
      }
    }
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int k = 2; k <= b.kl; k++)
      for (int j = 2; j <= b.jl; j++)
        for (int i = 2; i <= b.il; i++)
          for (int v = 0; v < 5; v++) b.DW(i, j, k, v) = b.DW(i, j, k, v) * (double)b.BL(i, j, k);
    if (lres) return MGE_OK;  // euler.f90:347-361
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int k = 2; k <= b.kl; k++)
      for (int j = 2; j <= b.jl; j++)
        for (int i = 2; i <= b.il; i++) {
          double de = fn * b.vdtim[b.I(i, j, k)] / b.vol;
          if (P.vt == 1) de = fn * b.dtim / b.vol;
          for (int v = 0; v < 5; v++) b.DW(i, j, k, v) = de * b.DW(i, j, k, v);
        }
    if (m % 2 != 0) {
      if (P.irs_variant == 1) psmoo_var(c, b);
      else psmoo_old(c, b);
    }
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int k = 2; k <= b.kl; k++)
      for (int j = 2; j <= b.jl; j++)
        for (int i = 2; i <= b.il; i++) {
          double lam = 1.0;
          if (unsteady && mgl == mlvl) {  // euler.f90:387-391
            double de = fn * b.vdtim[b.I(i, j, k)];
            if (P.vt == 1) de = fn * b.dtim;
            lam = 1.0 + de * 3.0 / 2.0 / P.dtstep;
          }
          for (int v = 0; v < 5; v++) b.W(i, j, k, v) = b.wn[v * N + b.I(i, j, k)] - b.DW(i, j, k, v) / lam;
          depvars_cell(P, b, i, j, k);
        }
    rc = bc_cutcell(c, b);
    if (rc) return rc;
    rc = bcond(c, b);
    if (rc) return rc;
  }
  if (nstage_limit > 0 && nstage_limit < P.mstage) return MGE_OK;
  // euler.f90:431-447
  if ((int)b.rtrms.size() <= ncyc) b.rtrms.resize(ncyc + 1, 0.0);
  double acc = 0.0;
  for (int k = 2; k <= b.kl; k++)
    for (int j = 2; j <= b.jl; j++)
      for (int i = 2; i <= b.il; i++) {
        double de = P.cfl * b.vdtim[b.I(i, j, k)];
        if (P.vt == 1) de = P.cfl * b.dtim;
        double rt = 0.0;
        if (b.BL(i, j, k) != 0) rt = b.DW(i, j, k, 0) / de;
        acc = acc + rt * rt;
      }
  b.rtrms[ncyc] = std::sqrt(acc / (double)((long)b.nx * b.ny * b.nz));
  return MGE_OK;
}

/* ------------------------------------------------------------------ grid transfer geometry */
/* Centre-based 2x2x2 stencil on the parent (coarse) grid for a point at
 * coarse coordinate u (cell q occupies [q-2, q-1)), clamped to [2, lc-1]. */
inline void coarse_stencil(double u, int lc, int& s, double& xi) {
  s = (int)std::floor(u + 1.5);
  if (s < 2) s = 2;
  if (s > lc - 1) s = lc - 1;
  xi = u + 1.5 - (double)s;
}
inline void trilinear_factor(double x, double y, double z, double* fac) {
  fac[0] = (1.0 - x) * (1.0 - y) * (1.0 - z);
  fac[1] = x * (1.0 - y) * (1.0 - z);
  fac[2] = (1.0 - x) * y * (1.0 - z);
  fac[3] = x * y * (1.0 - z);
  fac[4] = (1.0 - x) * (1.0 - y) * z;
  fac[5] = x * (1.0 - y) * z;
  fac[6] = (1.0 - x) * y * z;
  fac[7] = x * y * z;
}

/* collc.f90:58-158: restrict w and the volume-scaled residual of every child
 * (fine block at level mgl+1) onto coarse block b; sets marker. */
void collc(mgeo_ctx* c, OBlock& b) {
  std::fill(b.marker.begin(), b.marker.end(), 0);
  if ((int)c->lv.size() < b.level + 1) return;
  for (OBlock& f : c->lv[b.level]) {
    if (f.parent != b.serial) continue;
    int r[3] = {f.ratio[0], f.ratio[1], f.ratio[2]}, o[3] = {f.offset[0], f.offset[1], f.offset[2]};
    int n[3] = {f.nx / r[0], f.ny / r[1], f.nz / r[2]};
    int lf[3] = {f.il, f.jl, f.kl};
    for (int i = o[0] + 2; i <= o[0] + 1 + n[0]; i++) {
      if (i < 2 || i > b.il) continue;
      for (int j = o[1] + 2; j <= o[1] + 1 + n[1]; j++) {
        if (j < 2 || j > b.jl) continue;
        for (int k = o[2] + 2; k <= o[2] + 1 + n[2]; k++) {
          if (k < 2 || k > b.kl) continue;
          int ic[3] = {i, j, k}, sh[3];
          double xi[3];
          for (int d = 0; d < 3; d++) {
            // coarse centre in fine units: (q - 1.5 - o) * r ; fine centres at s - 1.5
            double t = ((double)ic[d] - 1.5 - (double)o[d]) * (double)r[d];
            int s = (int)std::floor(t + 1.5);
            if (s < 2) s = 2;
            if (s > lf[d] - 1) s = lf[d] - 1;
            sh[d] = s;
            xi[d] = t + 1.5 - (double)s;
          }
          double fac[8];
          trilinear_factor(xi[0], xi[1], xi[2], fac);
          size_t q = b.I(i, j, k);
          for (int v = 0; v < 5; v++) {
            double acc = 0.0;
            int nn = 0;
            for (int dk = 0; dk < 2; dk++)
              for (int dj = 0; dj < 2; dj++)
                for (int di = 0; di < 2; di++) {
                  double val = f.DW(sh[0] + di, sh[1] + dj, sh[2] + dk, v) / f.vol;
                  acc = acc + val * fac[nn++];
                }
            b.wr[v * b.N + q] = acc * b.vol;
            acc = 0.0;
            nn = 0;
            for (int dk = 0; dk < 2; dk++)
              for (int dj = 0; dj < 2; dj++)
                for (int di = 0; di < 2; di++) acc = acc + f.W(sh[0] + di, sh[1] + dj, sh[2] + dk, v) * fac[nn++];
            b.w[v * b.N + q] = acc;
          }
          b.marker[q] = 1;
        }
      }
    }
  }
}

/* Stencil of fine cell (i,j,k) of block f on its parent pb. Returns false
 * when the centre lies outside the parent's physical cells (eval_x2cell err). */
bool fine_to_coarse(const OBlock& f, const OBlock& pb, int i, int j, int k, int* sh, double* fac) {
  int ic[3] = {i, j, k};
  int lc[3] = {pb.il, pb.jl, pb.kl};
  int ncp[3] = {pb.nx, pb.ny, pb.nz};
  double xi[3];
  for (int d = 0; d < 3; d++) {
    double u = (double)f.offset[d] + ((double)ic[d] - 1.5) / (double)f.ratio[d];
    if (u < 0.0 || u >= (double)ncp[d]) return false;
    coarse_stencil(u, lc[d], sh[d], xi[d]);
  }
  trilinear_factor(xi[0], xi[1], xi[2], fac);
  return true;
}

/* addw.f90:83-188 */
void addw(mgeo_ctx* c, OBlock& f, int mgl, int mlvl) {
  if (f.parent < 1) return;
  OBlock& pb = c->lv[f.level - 2][f.parent - 1];
  std::vector<double> store_w = f.w;
  const bool fmg = (mgl - 1 == mlvl);
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int i = 2; i <= f.il; i++)
    for (int j = 2; j <= f.jl; j++)
      for (int k = 2; k <= f.kl; k++) {
        int sh[3];
        double fac[8];
        if (!fine_to_coarse(f, pb, i, j, k, sh, fac)) continue;
        size_t q = f.I(i, j, k);
        for (int v = 0; v < 5; v++) {
          double acc = 0.0;
          int nn = 0;
          for (int dk = 0; dk < 2; dk++)
            for (int dj = 0; dj < 2; dj++)
              for (int di = 0; di < 2; di++) {
                size_t cq = pb.I(sh[0] + di, sh[1] + dj, sh[2] + dk);
                double val = pb.w[v * pb.N + cq];
                if (!fmg) val = val - pb.ws[v * pb.N + cq];
                acc = acc + val * fac[nn++];
              }
          if (fmg) {
            if (f.blank[q] != 0) f.w[v * f.N + q] = acc;
          } else {
            if (f.blank[q] != 0) f.w[v * f.N + q] = store_w[v * f.N + q] + acc;
          }
        }
      }
}

/* bc_embed.f90:47-143: fine ghost cells from the parent level */
void bc_embed(mgeo_ctx* c, int lvl) {
  if (lvl <= 1) return;
  for (OBlock& f : c->lv[lvl - 1]) {
    if (f.parent < 1) continue;
    OBlock& pb = c->lv[lvl - 2][f.parent - 1];
    for (int i = 0; i <= f.ib; i++)
      for (int j = 0; j <= f.jb; j++)
        for (int k = 0; k <= f.kb; k++) {
          if (i >= 2 && i <= f.il && j >= 2 && j <= f.jl && k >= 2 && k <= f.kl) continue;
          int sh[3];
          double fac[8];
          if (!fine_to_coarse(f, pb, i, j, k, sh, fac)) continue;
          size_t q = f.I(i, j, k);
          if (f.blank[q] != 0) {
            for (int v = 0; v < 5; v++) {
              double acc = 0.0;
              int nn = 0;
              for (int dk = 0; dk < 2; dk++)
                for (int dj = 0; dj < 2; dj++)
                  for (int di = 0; di < 2; di++)
                    acc = acc + pb.w[v * pb.N + pb.I(sh[0] + di, sh[1] + dj, sh[2] + dk)] * fac[nn++];
              f.w[v * f.N + q] = acc;
            }
          }
          depvars_cell(c->prm, f, i, j, k);
        }
  }
}

/* Stencil of ghost cell (i,j,k) of block g on block p of the same level:
 * cell_center, eval_x2cell and shft_cell of bc_overlap.f90:63-73 (absent
 * helpers; the same construction as the prolongation's).  False when the
 * centre lies outside p's physical cells (eval_x2cell err). */
bool overlap_stencil(const OBlock& g, const OBlock& p, int i, int j, int k, int* sh, double* fac) {
  const int ic[3] = {i, j, k};
  const int lc[3] = {p.il, p.jl, p.kl};
  const int ncp[3] = {p.nx, p.ny, p.nz};
  double xi[3];
  for (int d = 0; d < 3; d++) {
    const double x = g.origin[d] + ((double)ic[d] - 1.5) * g.h[d];  // cell centre
    const double u = (x - p.origin[d]) / p.h[d];                     // in p's cells, 0 at its lower face
    if (u < 0.0 || u >= (double)ncp[d]) return false;
    coarse_stencil(u, lc[d], sh[d], xi[d]);
  }
  trilinear_factor(xi[0], xi[1], xi[2], fac);
  return true;
}

/* bc_overlap.f90:32-90: for every block of the level and every other block
 * it overlaps, the ghost cells (two layers) whose centre lies in the other
 * block's physical cells take the trilinear interpolation of its state,
 * then depvars.  Blocks and partners in serial order, cells i, j, k with k
 * innermost as the reference loops them; a ghost cell inside two partners
 * keeps the later one's value. */
void bc_overlap(mgeo_ctx* c, int lvl) {
  auto& L = c->lv[lvl - 1];
  if (L.size() < 2) return;
  for (OBlock& g : L)
    for (OBlock& p : L) {
      if (&g == &p) continue;
      for (int i = 0; i <= g.ib; i++)
        for (int j = 0; j <= g.jb; j++)
          for (int k = 0; k <= g.kb; k++) {
            if (i >= 2 && i <= g.il && j >= 2 && j <= g.jl && k >= 2 && k <= g.kl) continue;
            int sh[3];
            double fac[8];
            if (!overlap_stencil(g, p, i, j, k, sh, fac)) continue;
            for (int v = 0; v < 5; v++) {
              double acc = 0.0;
              int nn = 0;
              for (int dk = 0; dk < 2; dk++)
                for (int dj = 0; dj < 2; dj++)
                  for (int di = 0; di < 2; di++) acc = acc + p.W(sh[0] + di, sh[1] + dj, sh[2] + dk, v) * fac[nn++];
              g.W(i, j, k, v) = acc;
            }
            depvars_cell(c->prm, g, i, j, k);
          }
    }
}

int movco(mgeo_ctx* c, int mgl) {  // movco.f90:21-47
  if (mgl < 1 || mgl > (int)c->lv.size()) return fail(c, MGE_ENOTFOUND, "movco: bad level");
  for (OBlock& b : c->lv[mgl - 1]) {
    collc(c, b);
    depvars_all(c->prm, b);
    for (int i = 2; i <= b.il; i++)
      for (int j = 2; j <= b.jl; j++)
        for (int k = 2; k <= b.kl; k++)
          for (int v = 0; v < 5; v++) b.wn[v * b.N + b.I(i, j, k)] = b.W(i, j, k, v);
  }
  bc_overlap(c, mgl);
  for (OBlock& b : c->lv[mgl - 1]) {
    int rc = bcond(c, b);
    if (rc) return rc;
  }
  return MGE_OK;
}

int movfin(mgeo_ctx* c, int mgl, int mlvl) {  // movfin.f90:20-39
  if (mgl < 1 || mgl > (int)c->lv.size()) return fail(c, MGE_ENOTFOUND, "movfin: bad level");
  for (OBlock& b : c->lv[mgl - 1]) addw(c, b, mgl, mlvl);
  for (OBlock& b : c->lv[mgl - 1]) depvars_all(c->prm, b);
  bc_embed(c, mgl);
  bc_overlap(c, mgl);
  for (OBlock& b : c->lv[mgl - 1]) {
    int rc = bcond(c, b);
    if (rc) return rc;
  }
  return MGE_OK;
}

/* Wall forces from the cut-cell records (new; the reference has none):
   pressure on each wall face and, with NS, the wall's viscous stress.  The
   body takes the momentum the solver's wall flux gives the fluid, with the
   opposite sign: -(S*tau) for a solid on the + side, S*tau on the - side. */
/* whether a record's wall face counts: a face inside the physical cells of
   a block of lower serial on the same level is that block's (each once) */
bool record_counted(const mgeo_ctx* c, const OBlock& b, const int* ccid) {
  for (const OBlock& o : c->lv[b.level - 1]) {
    if (o.serial >= b.serial) continue;
    bool inside = true;
    const int n[3] = {o.nx, o.ny, o.nz};
    for (int d = 0; d < 3 && inside; d++) {
      const double x = b.origin[d] + ((double)ccid[d] - 1.5) * b.h[d];
      inside = x >= o.origin[d] && x < o.origin[d] + n[d] * o.h[d];
    }
    if (inside) return false;
  }
  return true;
}

void forces_block(mgeo_ctx* c, OBlock& b, const mge_solve_opts* o, double* F, double* M) {
  const double Sd[3] = {std::fabs(b.si[0]), std::fabs(b.sj[1]), std::fabs(b.sk[2])};
  for (const ORec& t : b.z) {
    if (!record_counted(c, b, t.ccid)) continue;
    int ax = t.zz - 1;
    double sgn = t.faceid >= 4 ? 1.0 : -1.0;
    double area = t.area;
    double pw = 0.5 * (b.P(t.ccid[0], t.ccid[1], t.ccid[2]) + t.psol);
    double fv[3] = {0, 0, 0};
    if (c->prm.eqntype == MGE_EQN_NS) {
      double vo[5];
      visc_wall(c->prm, b, t, Sd[ax], vo);
      for (int d = 0; d < 3; d++) fv[d] = t.faceid >= 4 ? -vo[1 + d] : vo[1 + d];
    }
    double f[3];
    for (int d = 0; d < 3; d++) f[d] = (d == ax ? pw * area * sgn : 0.0) + fv[d];
    double xf[3];
    int ic[3] = {t.ccid[0], t.ccid[1], t.ccid[2]};
    for (int d = 0; d < 3; d++) xf[d] = b.origin[d] + ((double)ic[d] - 1.5) * b.h[d];
    xf[ax] = xf[ax] + sgn * 0.5 * b.h[ax];
    double r[3];
    for (int d = 0; d < 3; d++) r[d] = xf[d] - (o ? o->moment_center[d] : 0.0);
    for (int d = 0; d < 3; d++) F[d] += f[d];
    M[0] += r[1] * f[2] - r[2] * f[1];
    M[1] += r[2] * f[0] - r[0] * f[2];
    M[2] += r[0] * f[1] - r[1] * f[0];
  }
  (void)c;
}

}  // namespace

/* ====================================================================== C API */
extern "C" {

void mgeo_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
int mgeo_get_threads(void) { return g_threads; }

int mgeo_init(const mge_params* prm, mgeo_ctx** out) {
  if (!prm || !out) return MGE_EBADCFG;
  mgeo_ctx* c = new mgeo_ctx();
  c->prm = *prm;
  if (prm->nlevel < 1 || prm->nlevel > MGE_MAX_LEVEL || prm->mstage < 1 || prm->mstage > MGE_MAX_STAGE) {
    delete c;
    return MGE_EBADCFG;
  }
  c->lv.resize(prm->nlevel);
  *out = c;
  return MGE_OK;
}

void mgeo_destroy(mgeo_ctx* c) { delete c; }
const char* mgeo_last_error(const mgeo_ctx* c) { return c ? c->err.c_str() : "null context"; }

int mgeo_add_block(mgeo_ctx* c, const mge_block_desc* d, int level, int serial) {
  if (level < 1 || level > (int)c->lv.size()) return fail(c, MGE_EBADCFG, "add_block: bad level");
  auto& L = c->lv[level - 1];
  if (serial != (int)L.size() + 1) return fail(c, MGE_EBADCFG, "add_block: serials must be added in order");
  if (d->nx < 2 || d->ny < 2 || d->nz < 2) return fail(c, MGE_EBADCFG, "add_block: need at least 2 cells per axis");
  L.emplace_back();
  OBlock& b = L.back();
  b.level = level;
  b.serial = serial;
  b.nx = d->nx; b.ny = d->ny; b.nz = d->nz;
  b.il = b.nx + 1; b.jl = b.ny + 1; b.kl = b.nz + 1;
  b.ie = b.il + 1; b.je = b.jl + 1; b.ke = b.kl + 1;
  b.ib = b.il + 2; b.jb = b.jl + 2; b.kb = b.kl + 2;
  b.Pi = b.ib + 1; b.Pj = b.jb + 1; b.Pk = b.kb + 1;
  b.N = b.Pi * b.Pj * b.Pk;
  for (int q = 0; q < 3; q++) {
    b.h[q] = d->h[q];
    b.origin[q] = d->origin[q];
    b.si[q] = d->si[q];
    b.sj[q] = d->sj[q];
    b.sk[q] = d->sk[q];
    b.ratio[q] = d->ratio[q];
    b.offset[q] = d->offset[q];
  }
  b.vol = d->cellvolume;
  for (int f = 0; f < 6; f++) {
    b.bctype[f] = d->bctype[f];
    for (int q = 0; q < 3; q++) b.fnv[f][q] = d->facenvec[f][q];
  }
  b.parent = d->parent;
  const size_t N = b.N;
  b.w.assign(5 * N, 0.0); b.p.assign(N, 0.0); b.wn.assign(5 * N, 0.0); b.ws.assign(5 * N, 0.0);
  if (c->prm.execmode == 1) { b.w1.assign(5 * N, 0.0); b.w2.assign(5 * N, 0.0); }  // make_flow.f90:38-39,60-61
  b.dw.assign(5 * N, 0.0); b.fw.assign(5 * N, 0.0); b.wr.assign(5 * N, 0.0); b.qf.assign(5 * N, 0.0);
  b.vdtim.assign(N, 0.0); b.radi.assign(N, 0.0); b.radj.assign(N, 0.0); b.radk.assign(N, 0.0);
  b.epsx.assign(N, 0.0); b.epsy.assign(N, 0.0); b.epsz.assign(N, 0.0);
  b.blank.assign(N, 1);
  b.marker.assign(N, 0);
  if (d->blank)
    for (size_t q = 0; q < N; q++) b.blank[q] = d->blank[q];
  b.z.resize(d->nmir);
  for (int m = 0; m < d->nmir; m++) {
    ORec& t = b.z[m];
    for (int q = 0; q < 3; q++) {
      t.ccid[q] = d->ccid[3 * m + q];
      t.scid[q] = d->scid[3 * m + q];
      t.nvec[q] = d->nvec[3 * m + q];
      t.qb[q] = d->qb ? d->qb[3 * m + q] : 0.0;
      t.psurf[q] = d->psurf ? d->psurf[3 * m + q] : 0.0;
      t.pnew[q] = t.psurf[q];
    }
    t.faceid = d->faceid[m];
    t.zz = d->zz[m];
    t.npoint = d->npoint[m];
    if (t.npoint < 0 || t.npoint > MGE_MAX_CLOUD) return fail(c, MGE_EBADCFG, "add_block: bad cloud size");
    for (int q = 0; q < MGE_MAX_CLOUD; q++) {
      t.coef[q] = d->coef[MGE_MAX_CLOUD * m + q];
      for (int e = 0; e < 3; e++) t.ijk[q][e] = d->ijkdex[(MGE_MAX_CLOUD * m + q) * 3 + e];
    }
    int ax = t.zz - 1;
    double fa = 1.0;
    for (int e = 0; e < 3; e++)
      if (e != ax) fa *= d->h[e];
    t.area = d->area ? d->area[m] : fa;
    t.psol = 0.0;
    for (int v = 0; v < 5; v++) t.wsol[v] = 0.0;
  }
  return MGE_OK;
}

int mgeo_commit(mgeo_ctx* c) {
  for (size_t l = 0; l < c->lv.size(); l++)
    if (c->lv[l].empty()) return fail(c, MGE_EBADCFG, "commit: a level has no block");
  c->committed = true;
  return MGE_OK;
}

int mgeo_init_flow(mgeo_ctx* c) {  // init_flow.f90:46-96 (free stream, no restart)
  const mge_params& P = c->prm;
  for (auto& L : c->lv)
    for (OBlock& b : L) {
      for (size_t q = 0; q < b.N; q++) {
        b.w[0 * b.N + q] = P.rho0;
        b.w[1 * b.N + q] = P.rho0 * P.u0;
        b.w[2 * b.N + q] = P.rho0 * P.v0;
        b.w[3 * b.N + q] = P.rho0 * P.w0;
        b.w[4 * b.N + q] = P.rho0 * P.h0 - P.p0;
      }
      depvars_all(P, b);
      int rc = bc_cutcell(c, b);
      if (rc) return rc;
      rc = bcond(c, b);
      if (rc) return rc;
      if (P.execmode == 1) {  // init_flow.f90:79-86
        b.w1 = b.w;
        b.w2 = b.w;
      }
    }
  c->itime = 0;
  return MGE_OK;
}

int mgeo_upload_state(mgeo_ctx* c, int level, int serial, const double* w) {
  OBlock* b = getb(c, level, serial);
  if (!b) return MGE_ENOTFOUND;
  std::memcpy(b->w.data(), w, 5 * b->N * sizeof(double));
  // init_flow.f90:46-66 after read_solut: depvars, bc_cutcell, bcond
  depvars_all(c->prm, *b);
  int rc = bc_cutcell(c, *b);
  if (rc) return rc;
  return bcond(c, *b);
}

int mgeo_download_field(mgeo_ctx* c, int level, int serial, const char* name, double* out, size_t count) {
  OBlock* b = getb(c, level, serial);
  if (!b) return MGE_ENOTFOUND;
  std::string n(name);
  const std::vector<double>* src = nullptr;
  if (n == "w") src = &b->w;
  else if (n == "p") src = &b->p;
  else if (n == "dw") src = &b->dw;
  else if (n == "fw") src = &b->fw;
  else if (n == "wn") src = &b->wn;
  else if (n == "ws") src = &b->ws;
  else if (n == "wr") src = &b->wr;
  else if (n == "qf") src = &b->qf;
  else if (n == "vdtim") src = &b->vdtim;
  else if (n == "w1" && !b->w1.empty()) src = &b->w1;
  else if (n == "w2" && !b->w2.empty()) src = &b->w2;
  if (src) {
    if (count < src->size()) return MGE_EBADCFG;
    std::memcpy(out, src->data(), src->size() * sizeof(double));
    return MGE_OK;
  }
  if (n == "eps") {  // epsx, epsy, epsz of the psmoo variant
    if (count < 3 * b->N) return fail(c, MGE_EBADCFG, "download_field: buffer too small");
    for (size_t q = 0; q < b->N; q++) {
      out[q] = b->epsx[q];
      out[b->N + q] = b->epsy[q];
      out[2 * b->N + q] = b->epsz[q];
    }
    return MGE_OK;
  }
  if (n == "lam") {
    if (count < b->N) return MGE_EBADCFG;
    for (size_t q = 0; q < b->N; q++) out[q] = b->radi[q] + b->radj[q] + b->radk[q];
    return MGE_OK;
  }
  if (n == "blank" || n == "marker") {
    if (count < b->N) return MGE_EBADCFG;
    const std::vector<int>& a = n == "blank" ? b->blank : b->marker;
    for (size_t q = 0; q < b->N; q++) out[q] = (double)a[q];
    return MGE_OK;
  }
  if (n == "wsol" || n == "psol") {
    size_t need = n == "wsol" ? 5 * b->z.size() : b->z.size();
    if (count < need) return MGE_EBADCFG;
    for (size_t m = 0; m < b->z.size(); m++) {
      if (n == "wsol")
        for (int v = 0; v < 5; v++) out[5 * m + v] = b->z[m].wsol[v];
      else
        out[m] = b->z[m].psol;
    }
    return MGE_OK;
  }
  if (n == "dtim") {
    out[0] = b->dtim;
    return MGE_OK;
  }
  return MGE_EBADCFG;
}

int mgeo_timestep(mgeo_ctx* c, int level, int serial) {
  OBlock* b = getb(c, level, serial);
  if (!b) return MGE_ENOTFOUND;
  return timestep(c, *b);
}

int mgeo_euler(mgeo_ctx* c, int level, int serial, int itime, int ncyc, int mgl, int mlvl, int lres, int lfir) {
  OBlock* b = getb(c, level, serial);
  if (!b) return MGE_ENOTFOUND;
  return euler(c, *b, itime, ncyc, mgl, mlvl, lres != 0, lfir != 0, 0);
}

int mgeo_euler_partial(mgeo_ctx* c, int level, int serial, int itime, int ncyc, int mgl, int mlvl, int lres,
                       int lfir, int nstage) {
  OBlock* b = getb(c, level, serial);
  if (!b) return MGE_ENOTFOUND;
  return euler(c, *b, itime, ncyc, mgl, mlvl, lres != 0, lfir != 0, nstage);
}

int mgeo_movco(mgeo_ctx* c, int mgl) { return movco(c, mgl); }
int mgeo_movfin(mgeo_ctx* c, int mgl, int mlvl) { return movfin(c, mgl, mlvl); }
int mgeo_bc_overlap(mgeo_ctx* c, int mgl) {
  if (mgl < 1 || mgl > (int)c->lv.size()) return MGE_ENOTFOUND;
  bc_overlap(c, mgl);
  return MGE_OK;
}

int mgeo_get_rtrms(mgeo_ctx* c, int level, int serial, int ncyc, double* out) {
  OBlock* b = getb(c, level, serial);
  if (!b) return MGE_ENOTFOUND;
  *out = (ncyc >= 0 && ncyc < (int)b->rtrms.size()) ? b->rtrms[ncyc] : 0.0;
  return MGE_OK;
}

/* upload_solut.f90:203-237 (called per block by blk2mgrid.f90:14-26): the
   cell-centre output variables rho, u, v, w, cp, mach, pt-loss (NS adds the
   energy re/rr and three zero gradients) of the physical cells, as
   solut(2:il,2:jl,2:kl,1:nval) in Fortran order */
int mgeo_upload_solut(mgeo_ctx* c, int level, int serial, double p_tot, double* out, size_t count, int* nval_out) {
  OBlock* b = getb(c, level, serial);
  if (!b) return MGE_ENOTFOUND;
  const mge_params& P = c->prm;
  const bool ns = P.eqntype == MGE_EQN_NS;
  const int nval = ns ? 11 : 7;
  if (nval_out) *nval_out = nval;
  const size_t nx = b->il - 1, ny = b->jl - 1, nz = b->kl - 1, ncell = nx * ny * nz;
  if (!out || count < nval * ncell) return MGE_EBADCFG;
  const double gamma = P.gamma;
  for (int k = 2; k <= b->kl; k++)
    for (int j = 2; j <= b->jl; j++)
      for (int i = 2; i <= b->il; i++) {
        const size_t q = b->I(i, j, k);
        const double rr = b->w[q];
        const double uu = b->w[b->N + q] / rr;
        const double vv = b->w[2 * b->N + q] / rr;
        const double ww = b->w[3 * b->N + q] / rr;
        const double re = b->w[4 * b->N + q];
        const double qq = 0.5 * (uu * uu + vv * vv + ww * ww) * rr;
        double pp = (gamma - 1.0) * fdim_(re, qq);
        const double mm = std::sqrt((uu * uu + vv * vv + ww * ww) / gamma / pp * rr);
        const double ptloss = pp * std::pow(1.0 + 0.2 * mm * mm, 3.5) / p_tot - 1.0;
        pp = (pp / P.p0 - 1.0) * 2.0 / (gamma * P.rm * P.rm);
        const size_t t = (i - 2) + nx * ((j - 2) + ny * (size_t)(k - 2));
        out[t] = rr;
        out[ncell + t] = uu;
        out[2 * ncell + t] = vv;
        out[3 * ncell + t] = ww;
        out[4 * ncell + t] = pp;
        out[5 * ncell + t] = mm;
        out[6 * ncell + t] = ptloss;
        if (ns) {
          out[7 * ncell + t] = re / rr;
          out[8 * ncell + t] = 0.0;
          out[9 * ncell + t] = 0.0;
          out[10 * ncell + t] = 0.0;
        }
      }
  return MGE_OK;
}

/* solver.f90:263-276,286: the end of a physical time step of the unsteady
   mode: w2 = w1, w1 = w on every block, and the step counter advances */
int mgeo_time_advance(mgeo_ctx* c, int* itime_out) {
  if (c->prm.execmode != 1) return fail(c, MGE_EBADCFG, "time_advance: execmode is not 1");
  for (auto& L : c->lv)
    for (OBlock& b : L) {
      b.w2 = b.w1;
      b.w1 = b.w;
    }
  c->itime += 1;
  if (itime_out) *itime_out = c->itime;
  return MGE_OK;
}

/* movsurf.f90:28-35 for one block, with bc_cutcell.f90:47-50's use of it:
   pnew = psurf + disp, the normal norv, the wall velocity vel/vel_fs */
int mgeo_move_surface(mgeo_ctx* c, int level, int serial, const double* disp, const double* norv,
                      const double* vel, double vel_fs) {
  OBlock* b = getb(c, level, serial);
  if (!b) return MGE_ENOTFOUND;
  if (!(vel_fs > 0.0)) return fail(c, MGE_EBADCFG, "move_surface: vel_fs must be positive");
  if (b->z.empty()) return MGE_OK;
  if (!disp || !norv || !vel) return fail(c, MGE_EBADCFG, "move_surface: null record array");
  for (size_t m = 0; m < b->z.size(); m++) {
    ORec& t = b->z[m];
    for (int q = 0; q < 3; q++) {
      t.pnew[q] = t.psurf[q] + disp[3 * m + q];
      t.nvec[q] = norv[3 * m + q];
      t.qb[q] = vel[3 * m + q] / vel_fs;
    }
  }
  return MGE_OK;
}

int mgeo_get_surface(mgeo_ctx* c, int level, int serial, double* pnew) {
  OBlock* b = getb(c, level, serial);
  if (!b || !pnew) return MGE_ENOTFOUND;
  for (size_t m = 0; m < b->z.size(); m++)
    for (int q = 0; q < 3; q++) pnew[3 * m + q] = b->z[m].pnew[q];
  return MGE_OK;
}

int mgeo_forces_compute(mgeo_ctx* c, int level, const mge_solve_opts* o, mge_forces* out) {
  if (level < 1 || level > (int)c->lv.size()) return MGE_ENOTFOUND;
  double F[3] = {0, 0, 0}, M[3] = {0, 0, 0};
  for (OBlock& b : c->lv[level - 1]) forces_block(c, b, o, F, M);
  const mge_params& P = c->prm;
  double qinf = 0.5 * P.rho0 * (P.u0 * P.u0 + P.v0 * P.v0 + P.w0 * P.w0);
  double aref = (o && o->ref_area > 0.0) ? o->ref_area : 1.0;
  double ed[3] = {std::cos(P.alpha) * std::cos(P.beta), std::sin(P.alpha) * std::cos(P.beta), std::sin(P.beta)};
  double el[3] = {-std::sin(P.alpha), std::cos(P.alpha), 0.0};
  for (int d = 0; d < 3; d++) {
    out->force[d] = F[d];
    out->moment[d] = M[d];
  }
  out->cd = (F[0] * ed[0] + F[1] * ed[1] + F[2] * ed[2]) / (qinf * aref);
  out->cl = (F[0] * el[0] + F[1] * el[1] + F[2] * el[2]) / (qinf * aref);
  return MGE_OK;
}

/* one multigrid cycle (solver.f90:126-234) at FMG level mlvl; returns max_res */
static int oracle_cycle(mgeo_ctx* c, int mlvl, int ncyc, double* max_res_out, double* ini_res_out) {
  const mge_params& P = c->prm;
  const int nlevel = (int)c->lv.size();
  std::vector<int> icyc(nlevel + 2, 0);
  const int itime = c->itime;
  int rc = 0;
  int mgl = mlvl;
  for (;;) {    // lopmg
    for (;;) {  // lopr
      icyc[mgl] += 1;
      bool lfir = (mgl != mlvl);
      for (OBlock& b : c->lv[mgl - 1]) {  // solver.f90:151-158
        if ((rc = timestep(c, b))) return rc;
        if ((rc = euler(c, b, itime, ncyc, mgl, mlvl, false, lfir, 0))) return rc;
        bc_overlap(c, mgl);
      }
      if (mgl == mlvl) {  // solver.f90:160-186
        double max_res = 1000.0;
        for (OBlock& b : c->lv[mgl - 1]) {
          double r = b.rtrms[ncyc];
          if (ncyc == 1 && ini_res_out) *ini_res_out = r;
          if (r < max_res) max_res = r;
          if (r != r) return fail(c, MGE_ENAN, "NaN residual (solver.f90:180)");
        }
        *max_res_out = max_res;
      }
      if (mlvl == 1) return MGE_OK;  // cycle lop0
      for (OBlock& b : c->lv[mgl - 1]) {  // solver.f90:197-201
        if ((rc = euler(c, b, itime, ncyc, mgl, mlvl, true, false, 0))) return rc;
        bc_overlap(c, mgl);
      }
      mgl = mgl - 1;
      if ((rc = movco(c, mgl))) return rc;
      if (mgl == 1) break;
    }
    bool lfir = true;
    for (;;) {  // lopp
      for (OBlock& b : c->lv[mgl - 1]) {  // solver.f90:215-222
        if ((rc = timestep(c, b))) return rc;
        if ((rc = euler(c, b, itime, ncyc, mgl, mlvl, false, lfir, 0))) return rc;
        bc_overlap(c, mgl);
      }
      lfir = false;
      mgl = mgl + 1;
      if ((rc = movfin(c, mgl, mlvl))) return rc;
      if (mgl == mlvl) return MGE_OK;   // exit lopmg
      if (icyc[mgl] != P.mgtype) break;  // cycle lopmg (W-cycle re-descent)
      icyc[mgl] = 0;
    }
  }
}

int mgeo_cycle(mgeo_ctx* c, int mlvl, int ncyc, double* max_res) {
  if (mlvl < 1 || mlvl > (int)c->lv.size() || !max_res) return MGE_EBADCFG;
  return oracle_cycle(c, mlvl, ncyc, max_res, nullptr);
}

/* solver.f90:109-292 (steady: execmode 0, one period, one step) */
int mgeo_solve(mgeo_ctx* c, const mge_solve_opts* o, double* hist, int hist_len, int* cycles_done,
               mge_forces* forces) {
  const mge_params& P = c->prm;
  const int nlevel = (int)c->lv.size();
  double max_res = 0.0, ini_res = 1.0;
  int nfin = 0, rc = 0;
  for (int mlvl = 1; mlvl <= nlevel; mlvl++) {
    for (int ncyc = 1; ncyc <= P.mcyc[mlvl - 1]; ncyc++) {
      if ((rc = oracle_cycle(c, mlvl, ncyc, &max_res, &ini_res))) return rc;
      if (mlvl == nlevel) {
        if (hist && nfin < hist_len) hist[nfin] = max_res;
        nfin++;
      }
      if (mlvl > 1) {  // solver.f90:237-239 (skipped by "cycle lop0" on the single-grid level)
        double drop = P.conv_drop > 0.0 ? P.conv_drop : 1.0e6;
        if (ini_res / max_res > drop) break;
      }
      if (o && o->max_cycles_total > 0 && mlvl == nlevel && nfin >= o->max_cycles_total) break;
    }
    if (mlvl < nlevel) {  // FMG prolongation, solver.f90:256-259
      if ((rc = movfin(c, mlvl + 1, mlvl))) return rc;
    }
  }
  if (cycles_done) *cycles_done = nfin;
  if (forces) mgeo_forces_compute(c, nlevel, o, forces);
  return MGE_OK;
}

}  // extern "C"
