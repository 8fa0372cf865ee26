// mge_kernels.cu -- sm_103a kernels of code_mge's multigrid Runge-Kutta cycle.
//
// GB300 executes FP64 at 1/58 of its FP32 rate (about 0.6 TFMA/s against
// 6.8 TB/s of HBM), so an all-FP64 JST stage is bound by FP64 issue, not by
// memory.  The stage is therefore split so that every per-cell and per-face
// quantity is evaluated exactly once (the reference re-evaluates each cell
// flux for both faces), with the intermediates kept in HBM/L2:
//
//   k_prep     per cell: 1/rho, rho*E+p, the cell flux F(w).s for i/j/k
//              (ceflux, eflux.f90:133-155) and the pressure sensors
//              (dflux.f90:71-76,131-136,188-193)
//   k_face     per face: averaged convective flux (eflux.f90:42-98) and the
//              blended 2nd/4th-difference dissipation (dflux.f90:82-112)
//   k_rec      per cut-cell record: the efluxb/dfluxb face replacements
//   k_combine  per cell: dw, fw, forcing, blanking, time-step scaling and,
//              without smoothing, the update + depvars (euler.f90:127-399)
//   k_irs_*    implicit residual smoothing lines (psmoo.f90:171-237), the
//              k-line fused with the update
//
// Arithmetic follows the reference expression by expression.  The plain path
// is compiled with --fmad=false (no contraction); divisions by a quantity
// whose reciprocal is already known use Markstein's correction
// (q0 = a*y, r = fma(-q0,b,a), q = fma(r,y,q0) with y = RN(1/b)), which
// returns the correctly rounded quotient (P. Markstein, IBM J. Res. Dev. 34,
// 1990), so results stay bit-identical to IEEE a/b at a third of its cost.
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include <cooperative_groups.h>
#include <algorithm>
#include <cstring>
#include <type_traits>

#include "exact_ops.cuh"
#include "fast_pow.cuh"
#include "mge_internal.h"
#include "soft_fp64.cuh"

namespace cg = cooperative_groups;

namespace mge {

// --------------------------------------------------------------- helpers
// a * b, for doubles on the integer pipes (soft_fp64.cuh: the same bits as
// the FP64 multiply), so that a kernel bound by the FP64 issue rate can move
// some of its independent products off the FP64 pipe
__device__ __forceinline__ double smul(double a, double b) { return soft::mul(a, b); }
__device__ __forceinline__ float smul(float a, float b) { return a * b; }
// a / b, for doubles on the integer pipes (the same bits as the FP64
// division, which costs about ten FP64 instructions)
__device__ __forceinline__ double sdiv(double a, double b) { return soft::div(a, b); }
__device__ __forceinline__ float sdiv(float a, float b) { return a / b; }
__device__ __forceinline__ double mdiv(double a, double b, double y) {
  double q = a * y;
  double r = fma(-q, b, a);
  return fma(r, y, q);
}
__device__ __forceinline__ float mdiv(float a, float b, float y) {
  float q = a * y;
  float r = fmaf(-q, b, a);
  return fmaf(r, y, q);
}
// mdiv with its first product on the integer pipes (smul, below): the same
// quotient
__device__ __forceinline__ double smul(double a, double b);
__device__ __forceinline__ double smdiv(double a, double b, double y) {
  double q = smul(a, y);
  double r = fma(-q, b, a);
  return fma(r, y, q);
}
__device__ __forceinline__ float smdiv(float a, float b, float y) { return mdiv(a, b, y); }
// reciprocals the host prepares once, RN(1/x) of the divisor x in the
// block's precision, so that mdiv gives the correctly rounded quotient
__device__ __forceinline__ double rcp_gm1(const PhysParams& P, double) { return P.rgm1; }
__device__ __forceinline__ float rcp_gm1(const PhysParams& P, float) { return P.rgm1f; }
__device__ __forceinline__ double rcp_gamma(const PhysParams& P, double) { return P.rgamma; }
__device__ __forceinline__ float rcp_gamma(const PhysParams& P, float) { return P.rgammaf; }
__device__ __forceinline__ double rcp_h(const DevBlock<double>& b, int d) { return b.rh[d]; }
__device__ __forceinline__ float rcp_h(const DevBlock<float>& b, int d) { return b.rhf[d]; }
__device__ __forceinline__ double rcp_4h(const DevBlock<double>& b, int d) { return b.r4h[d]; }
__device__ __forceinline__ float rcp_4h(const DevBlock<float>& b, int d) { return b.r4hf[d]; }
__device__ __forceinline__ double rcp_vol(const DevBlock<double>& b) { return b.rvol; }
__device__ __forceinline__ float rcp_vol(const DevBlock<float>& b) { return b.rvolf; }
// the line-sweep pivots in the sweep's precision (the FP32 sweeps read the
// single-precision tables: no conversion per cell)
__device__ __forceinline__ double irs_e1(const IrsTables& t, int q, double) { return t.e1[q]; }
__device__ __forceinline__ float irs_e1(const IrsTables& t, int q, float) { return t.e1f[q]; }
__device__ __forceinline__ double irs_e1r(const IrsTables& t, int q, double) { return t.e1r[q]; }
__device__ __forceinline__ float irs_e1r(const IrsTables& t, int q, float) { return t.e1rf[q]; }
__device__ __forceinline__ double irs_e2(const IrsTables& t, int q, double) { return t.e2[q]; }
__device__ __forceinline__ float irs_e2(const IrsTables& t, int q, float) { return t.e2f[q]; }
template <typename T> __device__ __forceinline__ T fdimT(T a, T b) { return a > b ? a - b : T(0); }
template <typename T> __device__ __forceinline__ T fmaxT(T a, T b) { return a > b ? a : b; }
template <typename T> __device__ __forceinline__ T fminT(T a, T b) { return a < b ? a : b; }

// depvars_one, depvars.f90:48-49
template <typename T> __device__ __forceinline__ T depvars(T gamma, const T* w) {
  // the products on the integer pipes and the halving as an exponent step:
  // the same bits as 0.5*(w1*w1 + w2*w2 + w3*w3)/w0 and (gamma-1)*dim(w4, qq)
  T qq = sdiv(mulhalf(smul(w[1], w[1]) + smul(w[2], w[2]) + smul(w[3], w[3])), w[0]);
  return smul(gamma - T(1), fdimT(w[4], qq));
}

struct Idx {
  int i, j, k;
};
__device__ __forceinline__ long long cidx(int Pi, int Pj, int i, int j, int k) {
  return (long long)i + (long long)Pi * ((long long)j + (long long)Pj * (long long)k);
}

inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

// --------------------------------------------------------------- timestep (timestep.f90:39-115)
// TC is the arithmetic precision (FP64 in the plain path, FP32 in the mixed one).
template <typename T, typename TC>
__device__ __forceinline__ unsigned long long body_timestep(const DevBlock<T>& b, const PhysParams& P, unsigned* err,
                                                            long long t) {
  const int nxl = b.nx, nyl = b.ny;
  unsigned long long mine = ~0ull;  // bits of this cell's vdtim for the global minimum
  int i = 2 + (int)(t % nxl);
  int j = 2 + (int)((t / nxl) % nyl);
  int k = 2 + (int)(t / ((long long)nxl * nyl));
  const long long N = b.N;
  const long long c = cidx(b.Pi, b.Pj, i, j, k);
  const TC gamma = (TC)P.gamma;
  TC w0 = (TC)b.w[c], w1 = (TC)b.w[N + c], w2 = (TC)b.w[2 * N + c], w3 = (TC)b.w[3 * N + c];
  TC pc = (TC)b.p[c];
  TC y = sdiv(TC(1), w0);
  TC cc = smdiv(smul(gamma, pc), w0, y);
  if (cc < TC(0) || cc != cc) {  // timestep.f90:45-48
    atomicCAS(err, 0u, (unsigned)ERR_NEGPRESS);  // the first stop in launch order wins
    return mine;
  }
  cc = sqrt(fmaxT(cc, TC(0)));
  TC uu = smdiv(w1, w0, y), uv = smdiv(w2, w0, y), uw = smdiv(w3, w0, y);
  // face vectors are axis-aligned: |u.s| = |u_d s_d|, |s| precomputed
  TC ri = fabs(smul(uu, (TC)b.s[0])) + smul(cc, (TC)b.sqrt_ds[0]);
  TC rj = fabs(smul(uv, (TC)b.s[1])) + smul(cc, (TC)b.sqrt_ds[1]);
  TC rk = fabs(smul(uw, (TC)b.s[2])) + smul(cc, (TC)b.sqrt_ds[2]);
  TC lsum = ri + rj + rk;
  TC fict;
  if (P.eqn_ns) {  // viscous spectral radii, timestep.f90:141-178
    const TC fmue = sdiv((TC)P.viscl, (TC)P.prlmean);
    const TC f1 = sdiv(sdiv(TC(4), w0), TC(3));
    const TC f2 = sdiv(gamma, w0);
    const TC fac = fmaxT(f1, f2);
    const TC dtv = sdiv(fac * fmue, (TC)b.vol);
    const TC s0 = (TC)b.s[0], s1 = (TC)b.s[1], s2 = (TC)b.s[2];
    TC rvi = dtv * (s0 * s0), rvj = dtv * (s1 * s1), rvk = dtv * (s2 * s2);
    fict = sdiv((TC)b.vol, lsum + (TC)P.cfac * (rvi + rvj + rvk));
  } else {
    fict = sdiv((TC)b.vol, lsum);
  }
  const TC plim = TC(0.001);
  TC pip = (TC)b.p[c + 1], pim = (TC)b.p[c - 1];
  TC pjp = (TC)b.p[c + b.Pi], pjm = (TC)b.p[c - b.Pi];
  long long pl = (long long)b.Pi * b.Pj;
  TC pkp = (TC)b.p[c + pl], pkm = (TC)b.p[c - pl];
  TC p2 = mul2(pc);
  TC dpi = fabs(sdiv(pip - p2 + pim, pip + p2 + pim + plim));
  TC dpj = fabs(sdiv(pjp - p2 + pjm, pjp + p2 + pjm + plim));
  TC dpk = fabs(sdiv(pkp - p2 + pkm, pkp + p2 + pkm + plim));
  TC r = sdiv(TC(1), TC(1) + fminT((TC)P.dimcfl, mul2(dpi + dpj + dpk)));
  if (P.unsteady) {  // timestep.f90:85-99,180-190: at most 2*dtstep/(3*cfl)
    const TC dtime = (TC(2) * (TC)P.dtstep) / (TC(3) * (TC)P.cfl);
    fict = fict < dtime ? fict : dtime;
  }
  TC vd = smul(fict, r);
  double vdd = (double)vd;
  if (vdd >= 0.0) mine = (unsigned long long)__double_as_longlong(vdd);
  if (b.blank[c] == 0) {  // timestep.f90:212-223
    b.vdtim[c] = T(0);
    b.lam[c] = T(0);
  } else {
    b.vdtim[c] = (T)vd;
    b.lam[c] = (T)lsum;
  }
  if (b.eps && P.smoo > 0.0) {
    // coefficients of the psmoo variant, timestep.f90:286-309; the radii of
    // blanked cells are zero there (timestep.f90:212-223), so their ratios
    // are 0/0 and the NaN-ignoring min/max give eps = smoo
    const bool bl = b.blank[c] == 0;
    const TC zi = bl ? TC(0) : ri, zj = bl ? TC(0) : rj, zk = bl ? TC(0) : rk;
    const TC smoo = (TC)P.smoo;
    const TC cflrat = sqrt(TC(1) + TC(4) * smoo);
    auto coef = [&](TC ra, TC rb, TC rc) -> TC {  // ra: this direction's radius
      TC reval = rb / ra + rc / ra;
      TC q = cflrat / (TC(1) + TC(0.0625) * reval);
      TC ex = TC(0.25) * (q * q - TC(1));
      ex = fmin(smoo, ex);
      return fmax(TC(0), ex);
    };
    b.eps[c] = (T)coef(zi, zj, zk);
    b.eps[N + c] = (T)coef(zj, zk, zi);
    b.eps[2 * N + c] = (T)coef(zk, zi, zj);
  }
  return mine;
}

// minimum over the calling block, then one atomicMin of its bits on dtim
// (vdtim >= 0, so the IEEE bit patterns order like the values); every thread
// of the block must call it
__device__ __forceinline__ void block_min_to(unsigned long long mine, double* dtim) {
  __shared__ unsigned long long smin[32];
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long q = __shfl_down_sync(0xffffffffu, mine, o);
    mine = q < mine ? q : mine;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) smin[wid] = mine;
  __syncthreads();
  if (wid == 0) {
    mine = (lane < (int)(blockDim.x >> 5)) ? smin[lane] : ~0ull;
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long q = __shfl_down_sync(0xffffffffu, mine, o);
      mine = q < mine ? q : mine;
    }
    if (lane == 0 && mine != ~0ull) atomicMin((unsigned long long*)dtim, mine);
  }
}

template <typename T, typename TC>
__global__ void k_timestep(DevBlock<T> b, PhysParams P, unsigned* err) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long mine = ~0ull;
  if (t < (long long)b.nx * b.ny * b.nz) mine = body_timestep<T, TC>(b, P, err, t);
  block_min_to(mine, b.dtim);  // global dtim (timestep.f90:112), kept even when vt = 0
}

template <typename T> __global__ void k_set_scalar(T* p, double v) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *p = (T)v;
}
// dtim travels as the bit pattern of a double (atomicMin on positive doubles)
__global__ void k_dtim_reset(double* p) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *p = 10.0;
}
template <typename T> __global__ void k_dtim_convert(double* src, T* dst) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *dst = (T)(*src);
}

// --------------------------------------------------------------- stage: per-cell pass
// Box [1..ie]x[1..je]x[1..ke]: every cell whose flux or sensor a face needs.
template <typename T>
__device__ __forceinline__ T van_albada(T a, T b, T e2);

// SLOPES: the MUSCL Roe form with the velocities of every cell already in
// F[0..2] (k_prim): the limited slope of each primitive variable along each
// direction goes to dlt[dir][var], once per cell.  A face takes the slope of
// its lower cell for the left state and that of its upper cell for the right
// state, the same van_albada(q(c)-q(c-1), q(c+1)-q(c)) it would form itself.
//
// FAST: the contracted form of the mixed precision's finest level (JST
// central scheme, Euler): the cell flux takes the velocity q = (w_d s)/rho
// once and multiplies, F(v) = q w(v), instead of rounding each product
// before its division.  The result is the same quantity to an FP64 rounding
// or two, not the reference's bit pattern.
template <typename T, bool SLOPES = false, bool FAST = false>
__device__ __forceinline__ void body_prep(const DevBlock<T>& b, const PhysParams& P, int dissip_on, long long t) {
  const int ex = b.ie, ey = b.je;  // count = ie (cells 1..ie)
  int i = 1 + (int)(t % ex);
  int j = 1 + (int)((t / ex) % ey);
  int k = 1 + (int)(t / ((long long)ex * ey));
  const long long N = b.N;
  const long long c = cidx(b.Pi, b.Pj, i, j, k);
  T w[5];
#pragma unroll
  for (int v = 0; v < 5; v++) w[v] = b.w[v * N + c];
  T p = b.p[c];
  T y = sdiv(T(1), w[0]);
  T Hc = w[4] + p;
  b.H[c] = Hc;
  if (P.eqn_ns && dissip_on) {  // velocity and temperature, zero in solid cells (euler.f90:140-154)
    const bool solid = b.blank[c] == 0;
#pragma unroll
    for (int a = 0; a < 3; a++) b.vt[a * N + c] = solid ? T(0) : mdiv(w[1 + a], w[0], y);
    b.vt[3 * N + c] = solid ? T(0) : sdiv(p, w[0] * (T)P.gas_const);
  }
  if (SLOPES) {
    const long long sts[3] = {1, (long long)b.Pi, (long long)b.Pi * b.Pj};
    // a face along d has physical tangential indices: only those cells need
    // the slope along d
    const bool ti = i >= 2 && i <= b.il, tj = j >= 2 && j <= b.jl, tk = k >= 2 && k <= b.kl;
    const bool need[3] = {tj && tk, ti && tk, ti && tj};
    auto prim = [&](long long q, int v) -> T {
      return v == 0 ? b.w[q] : (v == 4 ? b.p[q] : b.F[(long long)(v - 1) * N + q]);
    };
#pragma unroll
    for (int d = 0; d < 3; d++) {
      if (!need[d]) continue;
#pragma unroll
      for (int v = 0; v < 5; v++) {
        const T q0 = prim(c, v);
        const T dm = q0 - prim(c - sts[d], v), dp = prim(c + sts[d], v) - q0;
        b.dlt[(long long)(d * 5 + v) * N + c] = van_albada(dm, dp, (T)P.lim_e2[v]);
      }
    }
  }
  // the MUSCL Roe faces take their central flux from the reconstructed
  // states, not from the cell fluxes
  if (FAST) {
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const T s = (T)b.s[d];
      const T f0 = smul(w[1 + d], s);
      const T q = smul(f0, y);
      T f1 = smul(q, w[1]), f2 = smul(q, w[2]), f3 = smul(q, w[3]);
      if (d == 0) f1 = fma(p, s, f1);
      if (d == 1) f2 = fma(p, s, f2);
      if (d == 2) f3 = fma(p, s, f3);
      T* F = b.F + (long long)(d * 5) * N + c;
      F[0] = f0;
      F[N] = f1;
      F[2 * N] = f2;
      F[3 * N] = f3;
      F[4 * N] = smul(q, Hc);
    }
  } else if (P.distype != 2) {
#pragma unroll
    for (int d = 0; d < 3; d++) {
      // the products of this FP64-bound pass go to the integer pipes (smul);
      // the fused steps of the quotients stay on the FP64 pipe
      T s = (T)b.s[d];
      T f0 = smul(w[1 + d], s);  // sum(w(2:4)*ss) with the two zero components dropped
      T f1 = smdiv(smul(f0, w[1]), w[0], y);
      T f2 = smdiv(smul(f0, w[2]), w[0], y);
      T f3 = smdiv(smul(f0, w[3]), w[0], y);
      if (d == 0) f1 = f1 + smul(p, s);
      if (d == 1) f2 = f2 + smul(p, s);
      if (d == 2) f3 = f3 + smul(p, s);
      T f4 = smdiv(smul(f0, Hc), w[0], y);
      T* F = b.F + (long long)(d * 5) * N + c;
      F[0] = f0;
      F[N] = f1;
      F[2 * N] = f2;
      F[3 * N] = f3;
      F[4 * N] = f4;
    }
  }
  if (dissip_on && P.distype == 0) {
    // the differences the dissipation faces take (dflux.f90:95-99), once per
    // cell instead of once per face; the neighbour's enthalpy is formed
    // again with the same addition
    const long long sts[3] = {1, (long long)b.Pi, (long long)b.Pi * b.Pj};
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const long long cn = c - sts[d];
      T* Dl = b.dlt + (long long)(d * 5) * N + c;
#pragma unroll
      for (int v = 0; v < 4; v++) Dl[v * N] = w[v] - b.w[v * N + cn];
      Dl[4 * N] = Hc - (b.w[4 * N + cn] + b.p[cn]);
    }
  }
  if (dissip_on && P.distype == 0) {  // the pressure sensors of the JST faces
    const long long pl = (long long)b.Pi * b.Pj;
    // i: abs(p(i-1) +2p(i) +p(i+1)), dflux.f90:71-76
    {
      T pm = b.p[c - 1], pp = b.p[c + 1], p2 = mul2(p);
      T pb = fabs(pm + p2 + pp);
      b.fp[c] = (pb > T(0)) ? sdiv(fabs(pm - p2 + pp), pb) : T(0);
    }
    // j: abs(p(j+1) +2p(j) +p(j-1)), dflux.f90:131-136
    {
      T pm = b.p[c - b.Pi], pp = b.p[c + b.Pi], p2 = mul2(p);
      T pb = fabs(pp + p2 + pm);
      b.fp[N + c] = (pb > T(0)) ? sdiv(fabs(pp - p2 + pm), pb) : T(0);
    }
    // k: abs(p(k-1) +2p(k) +p(k+1)), dflux.f90:188-193
    {
      T pm = b.p[c - pl], pp = b.p[c + pl], p2 = mul2(p);
      T pb = fabs(pm + p2 + pp);
      b.fp[2 * N + c] = (pb > T(0)) ? sdiv(fabs(pm - p2 + pp), pb) : T(0);
    }
  }
}

// dflux_matrix, dflux.f90:283-339, with general face vector ss
template <typename T>
__device__ __noinline__ void dflux_matrix(T gamma, const T* u1, const T* u2, const T* dw, const T* ss, T* ff) {
  T gam1 = gamma - T(1), epsn = T(1), epsl = T(1);
  T rr = T(0.5) * (u1[0] + u2[0]);
  T us[3];
  for (int q = 0; q < 3; q++) us[q] = T(0.5) * (u1[q + 1] + u2[q + 1]) / rr;
  T ee = T(0.5) * (u1[4] + u2[4]) / rr;
  T qq = T(0.5) * (us[0] * us[0] + us[1] * us[1] + us[2] * us[2]);
  T c2 = gamma * gam1 * (ee - qq);
  T hh = c2 / gam1 + qq;
  T sss = ss[0] * ss[0] + ss[1] * ss[1] + ss[2] * ss[2];
  T cs = sqrt(c2 * sss);
  T qn = ss[0] * us[0] + ss[1] * us[1] + ss[2] * us[2];
  T e0 = fabs(qn) + cs;
  T e1 = fmaxT(epsn * e0, (T)fabs(qn + cs));
  T e2 = fmaxT(epsn * e0, (T)fabs(qn - cs));
  T e3 = fmaxT(epsl * e0, (T)fabs(qn));
  T s1 = T(0.5) * (e1 + e2), s2 = T(0.5) * (e1 - e2), s3 = e3;
  T ak1 = (s1 - s3) / c2 * gam1;
  T ak2 = s2 / cs;
  T ak3 = c2 / gam1 / sss;
  T d0 = dw[0], d1 = dw[1], d2 = dw[2], d3 = dw[3], d4 = dw[4];
  T vd = qq * d0 - us[0] * d1 - us[1] * d2 - us[2] * d3 + d4;
  T qd = qn * d0 - ss[0] * d1 - ss[1] * d2 - ss[2] * d3;
  ff[0] = ak1 * vd - ak2 * qd + s3 * d0;
  ff[1] = ak1 * (us[0] * vd - ss[0] * ak3 * qd) + ak2 * (gam1 * ss[0] * vd - us[0] * qd) + s3 * d1;
  ff[2] = ak1 * (us[1] * vd - ss[1] * ak3 * qd) + ak2 * (gam1 * ss[1] * vd - us[1] * qd) + s3 * d2;
  ff[3] = ak1 * (us[2] * vd - ss[2] * ak3 * qd) + ak2 * (gam1 * ss[2] * vd - us[2] * qd) + s3 * d3;
  ff[4] = ak1 * (hh * vd - qn * ak3 * qd) + ak2 * (gam1 * qn * vd - hh * qd) + s3 * d4;
}


// --------------------------------------------------------------- Roe, MUSCL and viscous faces
// (the reference's roepak/viscpak sources are not in its tree; these follow
// the published methods, as the oracle does: Roe 1981 with Harten's entropy
// fix, MUSCL with the van Albada limiter, central-gradient laminar stresses)
template <typename T>
__device__ __forceinline__ T van_albada(T a, T b, T e2) {
  // smooth form, no cut-off at a*b <= 0: with e2 > 0 a cut-off would make the
  // slope jump by up to b/3 when a changes sign.  Both differences zero (a
  // uniform stretch) and e2 > 0: the numerator is e2*a + e2*b, a zero with
  // the sign of a + b, and so is the quotient
  if (a == T(0) && b == T(0) && e2 > T(0)) return a + b;
  return sdiv((b * b + e2) * a + (a * a + e2) * b, a * a + b * b + T(2) * e2);
}

// yl, yr: RN(1/wl[0]) and RN(1/wr[0]); every quotient below that shares a
// divisor takes one reciprocal and mdiv, which rounds as the division does
template <typename T>
__device__ __noinline__ void roe_diss(const PhysParams& P, int d, T S, const T* wl, T pl, const T* wr, T pr, T yl, T yr,
                                      T* out) {
  const T g = (T)P.gamma;
  T ul[3], ur[3];
  for (int a = 0; a < 3; a++) {
    ul[a] = mdiv(wl[1 + a], wl[0], yl);
    ur[a] = mdiv(wr[1 + a], wr[0], yr);
  }
  T hl = mdiv(wl[4] + pl, wl[0], yl), hr = mdiv(wr[4] + pr, wr[0], yr);
  T rt = sqrt(mdiv(wr[0], wl[0], yl));
  T rh = rt * wl[0];
  const T den = T(1) + rt, yden = sdiv(T(1), den);
  T uh[3];
  for (int a = 0; a < 3; a++) uh[a] = mdiv(ul[a] + rt * ur[a], den, yden);
  T hh = mdiv(hl + rt * hr, den, yden);
  T q2 = uh[0] * uh[0] + uh[1] * uh[1] + uh[2] * uh[2];
  T c2 = (g - T(1)) * (hh - T(0.5) * q2);
  T ch = sqrt(fmaxT(c2, (T)1e-300));
  T un = uh[d];
  T dr = wr[0] - wl[0], dp = pr - pl, dun = ur[d] - ul[d];
  T du[3] = {ur[0] - ul[0], ur[1] - ul[1], ur[2] - ul[2]};
  T delta = (T)P.epsentr * (fabs(un) + ch);
  auto fix = [&](T lam) {
    T a = fabs(lam);
    return (a < delta && delta > T(0)) ? sdiv(lam * lam + delta * delta, T(2) * delta) : a;
  };
  T l1 = fix(un - ch), l2 = fix(un), l5 = fix(un + ch);
  const T c22 = T(2) * c2, yc22 = sdiv(T(1), c22);
  T a1 = mdiv(dp - rh * ch * dun, c22, yc22);
  T a2 = dr - sdiv(dp, c2);
  T a5 = mdiv(dp + rh * ch * dun, c22, yc22);
  T sh[3];
  for (int a = 0; a < 3; a++) sh[a] = rh * (du[a] - (a == d ? dun : T(0)));
  T k1[5], k5[5];
  k1[0] = T(1);
  k5[0] = T(1);
  for (int a = 0; a < 3; a++) {
    k1[1 + a] = uh[a] - (a == d ? ch : T(0));
    k5[1 + a] = uh[a] + (a == d ? ch : T(0));
  }
  k1[4] = hh - ch * un;
  k5[4] = hh + ch * un;
  T res[5];
  res[0] = l1 * a1 * k1[0] + l2 * a2 + l5 * a5 * k5[0];
  for (int a = 0; a < 3; a++) res[1 + a] = l1 * a1 * k1[1 + a] + l2 * (a2 * uh[a] + sh[a]) + l5 * a5 * k5[1 + a];
  res[4] = l1 * a1 * k1[4] + l2 * (a2 * T(0.5) * q2 + (uh[0] * sh[0] + uh[1] * sh[1] + uh[2] * sh[2])) + l5 * a5 * k5[4];
  for (int v = 0; v < 5; v++) out[v] = T(0.5) * S * res[v];
}

// face q (between q-1 and q) along D at cell c: cell states, MUSCL when order 2
template <typename T, int D>
__device__ __noinline__ void face_states(const DevBlock<T>& b, const PhysParams& P, long long c, int q, int order, T* wl, T* pl,
                            T* wr, T* pr) {
  const long long N = b.N;
  const long long st = D == 0 ? 1 : (D == 1 ? (long long)b.Pi : (long long)b.Pi * b.Pj);
  for (int v = 0; v < 5; v++) {
    wl[v] = b.w[v * N + c - st];
    wr[v] = b.w[v * N + c];
  }
  *pl = b.p[c - st];
  *pr = b.p[c];
  if (order < 2) return;
  const int lq = D == 0 ? b.il : (D == 1 ? b.jl : b.kl);
  if (q - 2 < 0 || q + 1 > lq + 2) return;
  if (b.blank[c - 2 * st] == 0 || b.blank[c - st] == 0 || b.blank[c] == 0 || b.blank[c + st] == 0) return;
  T qv[4][5];  // primitive (rho,u,v,w,p) at q-2..q+1
  for (int o = 0; o < 4; o++) {
    long long co = c + (o - 2) * st;
    T r = b.w[co], yr = sdiv(T(1), r);
    qv[o][0] = r;
    for (int a = 0; a < 3; a++) qv[o][1 + a] = mdiv(b.w[(1 + a) * N + co], r, yr);
    qv[o][4] = b.p[co];
  }
  T L[5], R[5];
  for (int kq = 0; kq < 5; kq++) {
    T dm = qv[1][kq] - qv[0][kq], d0 = qv[2][kq] - qv[1][kq], dp = qv[3][kq] - qv[2][kq];
    T e2 = (T)P.lim_e2[kq];
    L[kq] = qv[1][kq] + T(0.5) * van_albada(dm, d0, e2);
    R[kq] = qv[2][kq] - T(0.5) * van_albada(d0, dp, e2);
  }
  if (L[0] <= T(0) || R[0] <= T(0) || L[4] <= T(0) || R[4] <= T(0)) return;
  const T gm1 = (T)P.gamma - T(1), rg = rcp_gm1(P, T(0));
  wl[0] = L[0];
  wr[0] = R[0];
  for (int a = 0; a < 3; a++) {
    wl[1 + a] = L[0] * L[1 + a];
    wr[1 + a] = R[0] * R[1 + a];
  }
  wl[4] = mdiv(L[4], gm1, rg) + T(0.5) * L[0] * (L[1] * L[1] + L[2] * L[2] + L[3] * L[3]);
  wr[4] = mdiv(R[4], gm1, rg) + T(0.5) * R[0] * (R[1] * R[1] + R[2] * R[2] + R[3] * R[3]);
  *pl = L[4];
  *pr = R[4];
}

// y = RN(1/w[0])
// face_states in the MUSCL form from the per-cell velocities (F[0..2]) and
// limited slopes (dlt) of k_prim and the prep pass: the same values, with each
// quotient and slope formed once per cell instead of once per face
template <typename T, int D>
__device__ __noinline__ void face_states_pre(const DevBlock<T>& b, const PhysParams& P, long long c, int q, T* wl, T* pl,
                                             T* wr, T* pr) {
  const long long N = b.N;
  const long long st = D == 0 ? 1 : (D == 1 ? (long long)b.Pi : (long long)b.Pi * b.Pj);
  const long long cm = c - st;
  for (int v = 0; v < 5; v++) {
    wl[v] = b.w[v * N + cm];
    wr[v] = b.w[v * N + c];
  }
  *pl = b.p[cm];
  *pr = b.p[c];
  const int lq = D == 0 ? b.il : (D == 1 ? b.jl : b.kl);
  if (q - 2 < 0 || q + 1 > lq + 2) return;
  if (b.blank[c - 2 * st] == 0 || b.blank[cm] == 0 || b.blank[c] == 0 || b.blank[c + st] == 0) return;
  const T* S = b.dlt + (long long)(D * 5) * N;
  T L[5], R[5];
  L[0] = wl[0] + T(0.5) * S[cm];
  R[0] = wr[0] - T(0.5) * S[c];
  for (int a = 0; a < 3; a++) {
    L[1 + a] = b.F[(long long)a * N + cm] + T(0.5) * S[(long long)(1 + a) * N + cm];
    R[1 + a] = b.F[(long long)a * N + c] - T(0.5) * S[(long long)(1 + a) * N + c];
  }
  L[4] = *pl + T(0.5) * S[4 * N + cm];
  R[4] = *pr - T(0.5) * S[4 * N + c];
  if (L[0] <= T(0) || R[0] <= T(0) || L[4] <= T(0) || R[4] <= T(0)) return;
  const T gm1 = (T)P.gamma - T(1), rg = rcp_gm1(P, T(0));
  wl[0] = L[0];
  wr[0] = R[0];
  for (int a = 0; a < 3; a++) {
    wl[1 + a] = L[0] * L[1 + a];
    wr[1 + a] = R[0] * R[1 + a];
  }
  wl[4] = mdiv(L[4], gm1, rg) + T(0.5) * L[0] * (L[1] * L[1] + L[2] * L[2] + L[3] * L[3]);
  wr[4] = mdiv(R[4], gm1, rg) + T(0.5) * R[0] * (R[1] * R[1] + R[2] * R[2] + R[3] * R[3]);
  *pl = L[4];
  *pr = R[4];
}

template <typename T>
__device__ __forceinline__ void ceflux_gen(int D, const T* w, T p, T s, T y, T* f) {
  T f0 = w[1 + D] * s;
  f[0] = f0;
  f[1] = mdiv(f0 * w[1], w[0], y);
  f[2] = mdiv(f0 * w[2], w[0], y);
  f[3] = mdiv(f0 * w[3], w[0], y);
  f[1 + D] = f[1 + D] + p * s;
  f[4] = mdiv(f0 * (w[4] + p), w[0], y);
}

// laminar viscous flux through face q along D (at cell c), times S
template <typename T, int D>
__device__ __noinline__ void visc_face(const DevBlock<T>& b, const PhysParams& P, long long c, T S, T* out) {
  const long long N = b.N;
  const long long st[3] = {1, (long long)b.Pi, (long long)b.Pi * b.Pj};
  const long long cl = c - st[D];
  const double h[3] = {b.hx, b.hy, b.hz};
  T g[4][3];
  for (int a = 0; a < 4; a++) {
    const T* f = b.vt + (long long)a * N;
    for (int t = 0; t < 3; t++) {
      if (t == D)
        g[a][t] = mdiv(f[c] - f[cl], (T)h[D], rcp_h(b, D));
      else
        g[a][t] = mdiv((f[c + st[t]] - f[c - st[t]]) + (f[cl + st[t]] - f[cl - st[t]]), T(4) * (T)h[t],
                       rcp_4h(b, t));
    }
  }
  const T mu = (T)P.viscl, kt = (T)P.kt;
  T div = g[0][0] + g[1][1] + g[2][2];
  T tau[3];
  for (int a = 0; a < 3; a++) tau[a] = mu * (g[a][D] + g[D][a]) - (a == D ? (T(2) / T(3)) * mu * div : T(0));
  T uf[3];
  for (int a = 0; a < 3; a++) uf[a] = T(0.5) * (b.vt[a * N + cl] + b.vt[a * N + c]);
  out[0] = T(0);
  for (int a = 0; a < 3; a++) out[1 + a] = S * tau[a];
  out[4] = S * ((uf[0] * tau[0] + uf[1] * tau[1] + uf[2] * tau[2]) + kt * g[3][D]);
}

// --------------------------------------------------------------- stage: per-face pass
// Thread (i,j,k) in [2..ie]x[2..je]x[2..ke] owns the lower face of cell
// (i,j,k) in each direction whose tangential indices are physical.
// SCH: FACE_CENTRAL or FACE_ROE when the launch knows the scheme (each then
// gets its own register allocation), FACE_ANY to test P.distype; FACE_JST:
// the central scheme with scalar dissipation and no viscous flux, without
// the registers the matrix dissipation and the viscous face would take.
enum { FACE_CENTRAL = 0, FACE_ROE = 1, FACE_ANY = 2, FACE_JST = 3 };
template <typename T, int D, int SCH>
__device__ __forceinline__ void face_dir(const DevBlock<T>& b, const PhysParams& P, int dissip_on, T cd, int i, int j,
                                         int k) {
  const long long N = b.N;
  const long long st = D == 0 ? 1 : (D == 1 ? (long long)b.Pi : (long long)b.Pi * b.Pj);
  const long long c = cidx(b.Pi, b.Pj, i, j, k);
  const int q = D == 0 ? i : (D == 1 ? j : k);      // face between q-1 and q
  const int lq = D == 0 ? b.il : (D == 1 ? b.jl : b.kl);
  const int eq = lq + 1, bq = lq + 2;
  T* E = b.efs + (long long)(D * 5) * N;
  if (SCH != FACE_JST && P.eqn_ns && dissip_on) {  // viscous face flux, blended like the dissipation
    T o[5];
    visc_face<T, D>(b, P, c, (T)fabs(b.s[D]), o);
    T* V = b.vfs + (long long)(D * 5) * N;
#pragma unroll
    for (int v = 0; v < 5; v++) V[v * N + c] = cd * o[v];
  }
  const bool roe = SCH == FACE_ROE || (SCH == FACE_ANY && P.distype != 0);
  if (roe) {  // Roe: central part of the (reconstructed) states, upwind part into dfs
    T wl[5], wr[5], pl, pr;
    if (SCH == FACE_ROE && P.distype == 2)
      face_states_pre<T, D>(b, P, c, q, wl, &pl, wr, &pr);
    else
      face_states<T, D>(b, P, c, q, P.distype == 2 ? 2 : 1, wl, &pl, wr, &pr);
    const T yl = sdiv(T(1), wl[0]), yr = sdiv(T(1), wr[0]);
    if (P.distype == 2) {
      T f1[5], f2[5];
      ceflux_gen<T>(D, wr, pr, (T)b.s[D], yr, f1);
      ceflux_gen<T>(D, wl, pl, (T)b.s[D], yl, f2);
#pragma unroll
      for (int v = 0; v < 5; v++) E[v * N + c] = T(0.5) * (f1[v] + f2[v]);
    } else {
      const T* F = b.F + (long long)(D * 5) * N;
#pragma unroll
      for (int v = 0; v < 5; v++) E[v * N + c] = T(0.5) * (F[v * N + c] + F[v * N + c - st]);
    }
    if (!dissip_on) return;
    T o[5];
    roe_diss<T>(P, D, (T)fabs(b.s[D]), wl, pl, wr, pr, yl, yr, o);
    T* Df = b.dfs + (long long)(D * 5) * N;
#pragma unroll
    for (int v = 0; v < 5; v++) Df[v * N + c] = cd * o[v];
    return;
  }
  // convective: efs(q) = 0.5*(F(q) + F(q-1))
  const T* F = b.F + (long long)(D * 5) * N;
#pragma unroll
  for (int v = 0; v < 5; v++) E[v * N + c] = mulhalf(F[v * N + c] + F[v * N + c - st]);
  if (!dissip_on) return;
  // dissipation face q (dflux.f90:87-111)
  const T* fpd = b.fp + (long long)D * N;
  T f_m2 = (q - 2 == 0) ? T(0) : fpd[c - 2 * st];
  T f_m1 = fpd[c - st];
  T f_0 = fpd[c];
  T f_p1 = (q + 1 == bq) ? T(0) : fpd[c + st];
  // the sensors are >= +0: their maximum and the comparison below are taken
  // on the bit patterns (exact_ops.cuh)
  T ep = max_nonneg(max_nonneg(max_nonneg(f_m2, f_m1), f_0), f_p1);
  // lambda at ghost cells equals the adjacent physical cell (timestep.f90:227-282)
  long long cm = (q - 1 < 2) ? c : c - st;
  long long cp = (q > lq) ? c - st : c;
  T lam = mulhalf(b.lam[cm] + b.lam[cp]);
  T dis2 = (T)P.vis2 * ep;
  T dis4 = (T)P.vis4;
  dis4 = gt_nonneg(dis4, dis2) ? dis4 - dis2 : T(0);
  dis2 = dis2 * cd;
  dis4 = dis4 * cd;
  // diw(q) = w(q)-w(q-1), formed once per cell by the prep pass;
  // diw(1) = diw(2); diw(ib) = diw(ie)
  const T* Dl = b.dlt + (long long)(D * 5) * N;
  T out[5];
#pragma unroll
  for (int v = 0; v < 5; v++) {
    T d0 = Dl[v * N + c];
    T dm = (q - 1 == 1) ? d0 : Dl[v * N + c - st];
    T dp = (q + 1 == bq) ? d0 : Dl[v * N + c + st];
    T t3 = dp - mul2(d0) + dm;
    out[v] = smul(dis2, d0) - smul(dis4, t3);
  }
  if (SCH == FACE_JST || !P.matrix) {
#pragma unroll
    for (int v = 0; v < 5; v++) out[v] = smul(out[v], lam);
  } else {
    T ss[3] = {T(0), T(0), T(0)};
    ss[D] = (T)b.s[D];
    T ff[5], wq1[5], wq2[5];  // w at q-1 and q, enthalpy in slot 4
#pragma unroll
    for (int v = 0; v < 4; v++) {
      wq1[v] = b.w[v * N + c - st];
      wq2[v] = b.w[v * N + c];
    }
    wq1[4] = b.H[c - st];
    wq2[4] = b.H[c];
    dflux_matrix((T)P.gamma, wq1, wq2, out, ss, ff);
#pragma unroll
    for (int v = 0; v < 5; v++) out[v] = ff[v];
  }
  T* Df = b.dfs + (long long)(D * 5) * N;
#pragma unroll
  for (int v = 0; v < 5; v++) Df[v * N + c] = out[v];
  (void)eq;
}

template <typename T, int SCH = FACE_ANY>
__device__ __forceinline__ void body_face(const DevBlock<T>& b, const PhysParams& P, int dissip_on, T cd, long long t) {
  const int ex = b.ie - 1, ey = b.je - 1;  // 2..ie
  int i = 2 + (int)(t % ex);
  int j = 2 + (int)((t / ex) % ey);
  int k = 2 + (int)(t / ((long long)ex * ey));
  bool jp = j <= b.jl, kp = k <= b.kl, ip = i <= b.il;
  if (jp && kp) face_dir<T, 0, SCH>(b, P, dissip_on, cd, i, j, k);
  if (ip && kp) face_dir<T, 1, SCH>(b, P, dissip_on, cd, i, j, k);
  if (ip && jp) face_dir<T, 2, SCH>(b, P, dissip_on, cd, i, j, k);
}

// The contracted form's dissipation face (scalar JST, dflux.f90:87-112): the
// combine pass forms the convective part from the cell fluxes, so only dfs is
// written.  The face's coefficients take lambda once, dis2*lambda and
// dis4*lambda, and each variable is one product and two multiply-adds.
template <typename T, int D>
__device__ __forceinline__ void face_diss_fast(const DevBlock<T>& b, const PhysParams& P, T cd, int i, int j, int k) {
  const long long N = b.N;
  const long long st = D == 0 ? 1 : (D == 1 ? (long long)b.Pi : (long long)b.Pi * b.Pj);
  const long long c = cidx(b.Pi, b.Pj, i, j, k);
  const int q = D == 0 ? i : (D == 1 ? j : k);
  const int lq = D == 0 ? b.il : (D == 1 ? b.jl : b.kl);
  const int bq = lq + 2;
  const T* fpd = b.fp + (long long)D * N;
  const T f_m2 = (q - 2 == 0) ? T(0) : fpd[c - 2 * st];
  const T f_p1 = (q + 1 == bq) ? T(0) : fpd[c + st];
  const T ep = max_nonneg(max_nonneg(max_nonneg(f_m2, fpd[c - st]), fpd[c]), f_p1);
  const long long cm = (q - 1 < 2) ? c : c - st;
  const long long cp = (q > lq) ? c - st : c;
  const T lam = mulhalf(b.lam[cm] + b.lam[cp]);
  const T dis2 = smul((T)P.vis2, ep);
  const T dis4 = gt_nonneg((T)P.vis4, dis2) ? (T)P.vis4 - dis2 : T(0);
  const T a2 = smul(smul(dis2, cd), lam), a4 = smul(smul(dis4, cd), lam);
  const T* Dl = b.dlt + (long long)(D * 5) * N;
  T* Df = b.dfs + (long long)(D * 5) * N;
#pragma unroll
  for (int v = 0; v < 5; v++) {
    const T d0 = Dl[v * N + c];
    const T dm = (q - 1 == 1) ? d0 : Dl[v * N + c - st];
    const T dp = (q + 1 == bq) ? d0 : Dl[v * N + c + st];
    const T t3 = fma(T(-2), d0, dp + dm);
    Df[v * N + c] = fma(a2, d0, -smul(a4, t3));
  }
}

template <typename T>
__device__ __forceinline__ void body_face_diss(const DevBlock<T>& b, const PhysParams& P, T cd, long long t) {
  const int ex = b.ie - 1, ey = b.je - 1;  // 2..ie
  int i = 2 + (int)(t % ex);
  int j = 2 + (int)((t / ex) % ey);
  int k = 2 + (int)(t / ((long long)ex * ey));
  bool jp = j <= b.jl, kp = k <= b.kl, ip = i <= b.il;
  if (jp && kp) face_diss_fast<T, 0>(b, P, cd, i, j, k);
  if (ip && kp) face_diss_fast<T, 1>(b, P, cd, i, j, k);
  if (ip && jp) face_diss_fast<T, 2>(b, P, cd, i, j, k);
}

// --------------------------------------------------------------- stage: cut-cell record terms
// A record's corrections take dense face fluxes out and wall fluxes in.  The
// wall side depends only on the state (w, p, H, lambda, wsol, psol), not on
// this stage's face fluxes, so the record pass (rec_wall_terms) runs beside
// the face pass, and the combine pass takes the dense side from efs/dfs/vfs
// itself.  rec_wall holds per record (25 values):
//   [0,5)   efluxb first addend, [5,10) second addend (efluxb.f90:72-110)
//   [10,15) viscous wall stress term (NS)
//   [15,20) dfluxb Z0: fs1 - fs2 (JST) or the Roe wall flux
//   [20,25) dfluxb fs1 (solid on the + side) or fs2 (solid on the - side)
// With X the dense differences, dfluxb.f90 applies fw(t) = fw(t) - X and then
// fw(t) = fw(t) + Z at the cut cell (X0, Z0) and at its neighbour (X1, Z1).
template <typename T>
__device__ __forceinline__ void ceflux_axis(int D, const T* w, T p, T s, T* f) {
  T f0 = w[1 + D] * s;
  T y = T(1) / w[0];
  f[0] = f0;
  f[1] = mdiv(f0 * w[1], w[0], y);
  f[2] = mdiv(f0 * w[2], w[0], y);
  f[3] = mdiv(f0 * w[3], w[0], y);
  f[1 + D] = f[1 + D] + p * s;
  f[4] = mdiv(f0 * (w[4] + p), w[0], y);
}

template <typename T>
__device__ void rec_wall_terms(const DevBlock<T>& b, const PhysParams& P, int dissip_on, T cd, unsigned* err, int m) {
  T* W = b.rec_wall + 25LL * m;
  const long long N = b.N;
  const int* ri = b.rec_i + 8 * m;
  int i = ri[0], j = ri[1], k = ri[2], id = ri[3], zz = ri[4];
  int D = zz - 1;
  const long long st = D == 0 ? 1 : (D == 1 ? (long long)b.Pi : (long long)b.Pi * b.Pj);
  const long long c = cidx(b.Pi, b.Pj, i, j, k);
  T s = (T)b.s[D];
  T wc[5];
  for (int v = 0; v < 5; v++) wc[v] = b.w[v * N + c];
  if (fabs(wc[0]) < T(1.0e-8)) atomicCAS(err, 0u, (unsigned)ERR_ZERORHO);
  T psol = b.rec_psol[m];
  T wsol[5];
  for (int v = 0; v < 5; v++) wsol[v] = b.rec_wsol[5 * m + v];
  // efluxb.f90:66-110
  T f1[5], f2[5], f3[5];
  ceflux_axis<T>(D, wc, b.p[c], s, f1);
  ceflux_axis<T>(D, wsol, psol, s, f2);
  const bool plus = (id >= 4);  // solid on the + side
  long long cn = plus ? c - st : c + st;
  T wnb[5];
  for (int v = 0; v < 5; v++) wnb[v] = b.w[v * N + cn];
  ceflux_axis<T>(D, wnb, b.p[cn], s, f3);
  for (int v = 0; v < 5; v++) {
    T fs = T(0.5) * (f1[v] + f2[v]);
    T fa = T(0.5) * (f1[v] + f3[v]);
    W[v] = plus ? fa : fs;
    W[5 + v] = plus ? fs : fa;
  }
  if (!dissip_on) return;
  if (P.eqn_ns) {  // no-slip adiabatic wall face: normal gradients to the mirror state only
    T u[3], ug[3], qbv[3] = {(T)b.rec_qb[3 * m], (T)b.rec_qb[3 * m + 1], (T)b.rec_qb[3 * m + 2]};
    const double hh[3] = {b.hx, b.hy, b.hz};
    for (int a = 0; a < 3; a++) {
      u[a] = wc[1 + a] / wc[0];
      ug[a] = T(2) * qbv[a] - u[a];
    }
    const T mu = (T)P.viscl, S = (T)fabs(b.s[D]);
    T o[5];
    T tau[3];
    for (int a = 0; a < 3; a++) {
      T gn = plus ? (ug[a] - u[a]) / (T)hh[D] : (u[a] - ug[a]) / (T)hh[D];
      tau[a] = (a == D) ? (T(4) / T(3)) * mu * gn : mu * gn;
    }
    o[0] = T(0);
    for (int a = 0; a < 3; a++) o[1 + a] = S * tau[a];
    o[4] = S * (qbv[0] * tau[0] + qbv[1] * tau[1] + qbv[2] * tau[2]);
    for (int v = 0; v < 5; v++) W[10 + v] = plus ? -(cd * o[v]) : cd * o[v];
  }
  if (P.distype != 0) {  // Roe: the wall face's upwind flux taken to the ghost state
    T o[5];
    const T S = (T)fabs(b.s[D]);
    const T yc = T(1) / wc[0], ys = T(1) / wsol[0];
    if (plus)
      roe_diss<T>(P, D, S, wc, b.p[c], wsol, psol, yc, ys, o);
    else
      roe_diss<T>(P, D, S, wsol, psol, wc, b.p[c], ys, yc, o);
    for (int v = 0; v < 5; v++) W[15 + v] = plus ? -(cd * o[v]) : cd * o[v];
    return;
  }
  // dfluxb.f90:29-423; w(:,5) is the enthalpy here
  wsol[4] = wsol[4] + psol;
  auto pp = [&](int a) -> T { return b.p[c + a * st]; };
  // the enthalpy formed here with the prep pass's addition: a record at the
  // block's edge reaches the outer ghost layer, where the prep pass forms no H
  auto ww = [&](int a, int v) -> T {
    const long long q = c + a * st;
    return v < 4 ? b.w[v * N + q] : b.w[4 * N + q] + b.p[q];
  };
  auto lamc = [&](int a) -> T {
    // lambda with the ghost-copy rule of timestep.f90:227-282 along the record axis
    int q = (D == 0 ? i : (D == 1 ? j : k)) + a;
    int lq = D == 0 ? b.il : (D == 1 ? b.jl : b.kl);
    int qq = q < 2 ? 2 : (q > lq ? lq : q);
    return b.lam[c + (long long)(qq - (q - a)) * st];
  };
  const int pos = D == 0 ? i : (D == 1 ? j : k);
  const int lim = D == 0 ? b.ib : (D == 1 ? b.jb : b.kb);
  T fp[3], ep, lam, dis2, dis4;
  T fs1[5], fs2[5], diw[3][5];
  T ssv[3] = {T(0), T(0), T(0)};
  ssv[D] = s;
  auto setdis = [&]() {
    dis2 = (T)P.vis2 * ep;
    dis4 = (T)P.vis4;
    dis4 = fdimT(dis4, dis2);
    dis2 = dis2 * cd;
    dis4 = dis4 * cd;
  };
  if (plus) {
    if (D == 0) {
      fp[0] = fabs(pp(-2) - T(2) * pp(-1) + pp(0)) / fabs(pp(-2) + T(2) * pp(-1) + pp(0));
      fp[1] = fabs(pp(-1) - T(2) * pp(0) + psol) / fabs(pp(-1) + T(2) * pp(0) + psol);
    } else {
      fp[0] = fabs(pp(0) - T(2) * pp(-1) + pp(-2)) / fabs(pp(0) + T(2) * pp(-1) + pp(-2));
      fp[1] = fabs(psol - T(2) * pp(0) + pp(-1)) / fabs(psol + T(2) * pp(0) + pp(-1));
    }
    ep = fmaxT(fp[0], fp[1]);
    lam = lamc(0);
    setdis();
    for (int v = 0; v < 5; v++) {
      diw[0][v] = ww(0, v) - ww(-1, v);
      diw[1][v] = wsol[v] - ww(0, v);
      diw[2][v] = diw[1][v];
      fs2[v] = diw[2][v] - T(2) * diw[1][v] + diw[0][v];
      fs2[v] = dis2 * diw[1][v] - dis4 * fs2[v];
    }
    if (!P.matrix) {
      for (int v = 0; v < 5; v++) fs2[v] = fs2[v] * lam;
    } else {
      T wcv[5], tmp[5];
      for (int v = 0; v < 5; v++) wcv[v] = ww(0, v);
      dflux_matrix((T)P.gamma, wcv, wsol, fs2, ssv, tmp);
      for (int v = 0; v < 5; v++) fs2[v] = tmp[v];
    }
    if (pos - 3 >= 0)
      fp[2] = fabs(pp(-1) - T(2) * pp(-2) + pp(-3)) / fabs(pp(-1) + T(2) * pp(-2) + pp(-3));
    else
      fp[2] = T(0);
    ep = fmaxT(fmaxT(fp[0], fp[1]), fp[2]);
    lam = T(0.5) * (lamc(-1) + lamc(0));
    setdis();
    for (int v = 0; v < 5; v++) {
      diw[0][v] = ww(-1, v) - ww(-2, v);
      diw[1][v] = ww(0, v) - ww(-1, v);
      diw[2][v] = wsol[v] - ww(0, v);
      fs1[v] = diw[2][v] - T(2) * diw[1][v] + diw[0][v];
      fs1[v] = dis2 * diw[1][v] - dis4 * fs1[v];
    }
    if (!P.matrix) {
      for (int v = 0; v < 5; v++) fs1[v] = fs1[v] * lam;
    } else {
      T wa[5], wcv[5], tmp[5];
      for (int v = 0; v < 5; v++) {
        wa[v] = ww(-1, v);
        wcv[v] = ww(0, v);
      }
      dflux_matrix((T)P.gamma, wa, wcv, fs1, ssv, tmp);
      for (int v = 0; v < 5; v++) fs1[v] = tmp[v];
    }
    for (int v = 0; v < 5; v++) {
      W[15 + v] = fs1[v] - fs2[v];
      W[20 + v] = fs1[v];
    }
  } else {
    fp[0] = fabs(pp(1) - T(2) * pp(0) + psol) / fabs(pp(1) + T(2) * pp(0) + psol);
    fp[1] = fabs(pp(2) - T(2) * pp(1) + pp(0)) / fabs(pp(2) + T(2) * pp(1) + pp(0));
    if (pos + 3 <= lim)
      fp[2] = fabs(pp(3) - T(2) * pp(2) + pp(1)) / fabs(pp(3) + T(2) * pp(2) + pp(1));
    else
      fp[2] = T(0);
    ep = fmaxT(fmaxT(fp[0], fp[1]), fp[2]);
    lam = T(0.5) * (lamc(0) + lamc(1));
    setdis();
    for (int v = 0; v < 5; v++) {
      diw[0][v] = ww(0, v) - wsol[v];
      diw[1][v] = ww(1, v) - ww(0, v);
      diw[2][v] = ww(2, v) - ww(1, v);
      fs2[v] = diw[2][v] - T(2) * diw[1][v] + diw[0][v];
      fs2[v] = dis2 * diw[1][v] - dis4 * fs2[v];
    }
    if (!P.matrix) {
      for (int v = 0; v < 5; v++) fs2[v] = fs2[v] * lam;
    } else {
      T wcv[5], wbv[5], tmp[5];
      for (int v = 0; v < 5; v++) {
        wcv[v] = ww(0, v);
        wbv[v] = ww(1, v);
      }
      dflux_matrix((T)P.gamma, wcv, wbv, fs2, ssv, tmp);
      for (int v = 0; v < 5; v++) fs2[v] = tmp[v];
    }
    ep = fmaxT(fp[0], fp[1]);
    lam = lamc(0);
    setdis();
    for (int v = 0; v < 5; v++) {
      diw[1][v] = ww(0, v) - wsol[v];
      diw[0][v] = diw[1][v];
      diw[2][v] = ww(1, v) - ww(0, v);
      fs1[v] = diw[2][v] - T(2) * diw[1][v] + diw[0][v];
      fs1[v] = dis2 * diw[1][v] - dis4 * fs1[v];
    }
    if (!P.matrix) {
      for (int v = 0; v < 5; v++) fs1[v] = fs1[v] * lam;
    } else {
      T wcv[5], tmp[5];
      for (int v = 0; v < 5; v++) wcv[v] = ww(0, v);
      dflux_matrix((T)P.gamma, wsol, wcv, fs1, ssv, tmp);
      for (int v = 0; v < 5; v++) fs1[v] = tmp[v];
    }
    for (int v = 0; v < 5; v++) {
      W[15 + v] = fs1[v] - fs2[v];
      W[20 + v] = fs2[v];
    }
  }
}

template <typename T>
__global__ void k_rec_wall(DevBlock<T> b, PhysParams P, int dissip_on, T cd, unsigned* err) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m < b.nmir) rec_wall_terms(b, P, dissip_on, cd, err, m);
}

// the record's geometry: cell, axis stride, solid side
template <typename T>
__device__ __forceinline__ void rec_geom(const DevBlock<T>& b, int m, long long& c, long long& st, int& D, bool& plus) {
  const int* ri = b.rec_i + 8 * m;
  D = ri[4] - 1;
  st = D == 0 ? 1 : (D == 1 ? (long long)b.Pi : (long long)b.Pi * b.Pj);
  c = cidx(b.Pi, b.Pj, ri[0], ri[1], ri[2]);
  plus = ri[3] >= 4;
}

// --------------------------------------------------------------- stage: combine + update
// euler.f90:320-331,387-391: the unsteady mode's factor lam = 1 + 3*de/(2*dtstep)
// with de = fn*vdtim (or fn*dtim), dividing the coarse-level residual and the
// finest level's update
template <typename T>
__device__ __forceinline__ T unsteady_lam(const DevBlock<T>& b, const PhysParams& P, const StageArgs& A, long long c) {
  const T vd = A.vt ? (T)(*b.dtim) : b.vdtim[c];
  const T de = (T)A.fn * vd;
  return T(1) + ((de * T(3)) / T(2)) / (T)P.dtstep;
}

// The cut-cell records act here in record order on the cell they touch: the
// dense face pair out, the wall pair in, from this stage's face fluxes and
// the record pass's wall terms (rec_wall_terms).
//
// FAST (the contracted form, JST central scheme): the convective part of dw
// is the central difference of the cell fluxes, efs(q) - efs(q+1) =
// 0.5*(F(q-1) - F(q+1)) in each direction, so no convective face pass runs;
// a record's dense face pair takes the same difference.
template <typename T, bool FAST = false>
__device__ __forceinline__ void body_combine(const DevBlock<T>& b, const PhysParams& P, const StageArgs& A,
                                             unsigned* err, long long t) {
  const int nxl = b.nx, nyl = b.ny;
  int i = 2 + (int)(t % nxl);
  int j = 2 + (int)((t / nxl) % nyl);
  int k = 2 + (int)(t / ((long long)nxl * nyl));
  const long long N = b.N;
  const long long c = cidx(b.Pi, b.Pj, i, j, k);
  const long long sj = b.Pi, sk = (long long)b.Pi * b.Pj;
  const int tg = b.cutmap[c];
  T dwv[5], fwv[5];
  if (FAST) {
    const T* Fx = b.F;
    const T* Fy = b.F + 5 * N;
    const T* Fz = b.F + 10 * N;
#pragma unroll
    for (int v = 0; v < 5; v++) {
      const T a = (Fx[v * N + c - 1] - Fx[v * N + c + 1]) + (Fy[v * N + c - sj] - Fy[v * N + c + sj]);
      dwv[v] = mulhalf(a + (Fz[v * N + c - sk] - Fz[v * N + c + sk]));
    }
  } else {
    const T* Ex = b.efs;
    const T* Ey = b.efs + 5 * N;
    const T* Ez = b.efs + 10 * N;
#pragma unroll
    for (int v = 0; v < 5; v++) {
      T a = Ex[v * N + c] - Ex[v * N + c + 1];
      a = a + Ey[v * N + c] - Ey[v * N + c + sj];
      a = a + Ez[v * N + c] - Ez[v * N + c + sk];
      dwv[v] = a;
    }
  }
  // fw: blending and dissipation (euler.f90:127-135, dflux.f90:116-238)
  const T fac = T(1) - (T)A.cd;
  if (A.dissip_on) {
    const T* Dx = b.dfs;
    const T* Dy = b.dfs + 5 * N;
    const T* Dz = b.dfs + 10 * N;
    T vis[5];
#pragma unroll
    for (int v = 0; v < 5; v++) vis[v] = A.scale_fw ? smul(b.fw[v * N + c], fac) : T(0);
    if (P.eqn_ns) {  // viscous faces, then the viscous wall faces in record order
      const T* Vx = b.vfs;
      const T* Vy = b.vfs + 5 * N;
      const T* Vz = b.vfs + 10 * N;
#pragma unroll
      for (int v = 0; v < 5; v++) {
        T a = vis[v];
        a = a + (Vx[v * N + c] - Vx[v * N + c + 1]);
        a = a + (Vy[v * N + c] - Vy[v * N + c + sj]);
        a = a + (Vz[v * N + c] - Vz[v * N + c + sk]);
        vis[v] = a;
      }
      if (tg >= 0) {
        for (int o = b.tgt_off[tg]; o < b.tgt_off[tg + 1]; o++) {
          const int op = b.tgt_ops[o];
          if (op & 1) continue;
          const int m = op >> 1;
          long long cm, st;
          int D;
          bool plus;
          rec_geom(b, m, cm, st, D, plus);
          const T* V = b.vfs + (long long)(D * 5) * N;
          const T* Wm = b.rec_wall + 25LL * m;
          const long long qn = plus ? cm + st : cm;  // the wall face's upper cell
#pragma unroll
          for (int v = 0; v < 5; v++) {
            const T x = plus ? -V[v * N + qn] : V[v * N + qn];
            vis[v] = vis[v] - x;
            vis[v] = vis[v] + Wm[10 + v];
          }
        }
      }
    }
    if (FAST) {
#pragma unroll
      for (int v = 0; v < 5; v++) {
        const T a = (Dx[v * N + c] - Dx[v * N + c + 1]) + (Dy[v * N + c] - Dy[v * N + c + sj]);
        const T d = a + (Dz[v * N + c] - Dz[v * N + c + sk]);
        fwv[v] = A.scale_fw ? fma(b.fw[v * N + c], fac, d) : d;
      }
    } else {
#pragma unroll
      for (int v = 0; v < 5; v++) {
        T a = vis[v];
        a = a + (Dx[v * N + c] - Dx[v * N + c + 1]);
        a = a + (Dy[v * N + c] - Dy[v * N + c + sj]);
        a = a + (Dz[v * N + c] - Dz[v * N + c + sk]);
        fwv[v] = a;
      }
    }
  } else {
#pragma unroll
    for (int v = 0; v < 5; v++) fwv[v] = A.scale_fw ? smul(b.fw[v * N + c], fac) : T(0);
  }
  if (tg >= 0) {
    // cut-cell wall faces, this cell's records in record order: efluxb on dw
    // (efluxb.f90:72-110) and dfluxb on fw (dfluxb.f90:47-420)
    for (int o = b.tgt_off[tg]; o < b.tgt_off[tg + 1]; o++) {
      const int op = b.tgt_ops[o];
      const int m = op >> 1;
      long long cm, st;
      int D;
      bool plus;
      rec_geom(b, m, cm, st, D, plus);
      const T* Wm = b.rec_wall + 25LL * m;
      if (!(op & 1)) {  // efluxb on the cut cell: the dense face pair out, the wall pair in
        const T* E = b.efs + (long long)(D * 5) * N;
        const T* Fd = b.F + (long long)(D * 5) * N;
#pragma unroll
        for (int v = 0; v < 5; v++) {
          const T x = FAST ? mulhalf(Fd[v * N + cm - st] - Fd[v * N + cm + st]) : E[v * N + cm] - E[v * N + cm + st];
          dwv[v] = dwv[v] - x;
          dwv[v] = dwv[v] + Wm[v] - Wm[5 + v];
        }
      }
      if (A.dissip_on) {
        const T* Dd = b.dfs + (long long)(D * 5) * N;
        auto dd = [&](int a, int v) -> T { return Dd[v * N + cm + a * st]; };
#pragma unroll
        for (int v = 0; v < 5; v++) {
          T x, z;
          if (P.distype != 0) {  // Roe wall: the dense face out, the ghost-state flux in (neighbour: zeros)
            const long long qn = plus ? cm + st : cm;
            x = (op & 1) ? T(0) : (plus ? -Dd[v * N + qn] : Dd[v * N + qn]);
            z = (op & 1) ? T(0) : Wm[15 + v];
          } else if (!(op & 1)) {  // dfluxb X0, Z0
            x = dd(0, v) - dd(1, v);
            z = Wm[15 + v];
          } else if (plus) {  // dfluxb X1, Z1, solid on the + side
            x = dd(-1, v) - dd(0, v);
            z = dd(-1, v) - Wm[20 + v];
          } else {  // solid on the - side
            x = dd(1, v) - dd(2, v);
            z = Wm[20 + v] - dd(2, v);
          }
          fwv[v] = fwv[v] - x;
          fwv[v] = fwv[v] + z;
        }
      }
    }
  }
  if (A.dissip_on || A.scale_fw) {
#pragma unroll
    for (int v = 0; v < 5; v++) b.fw[v * N + c] = fwv[v];
  }
#pragma unroll
  for (int v = 0; v < 5; v++) dwv[v] = dwv[v] + fwv[v];
  if (A.tmode) {  // euler.f90:249-275: BDF2, or the first step's (halved) BDF1
    const T f = (T(0.5) * (T)b.vol) / (T)P.dtstep;
#pragma unroll
    for (int v = 0; v < 5; v++) {
      const T wv = b.w[v * N + c], w1 = b.w1[v * N + c];
      const T d = A.tmode == 2 ? (T(3) * wv - T(4) * w1) + b.w2[v * N + c] : wv - w1;
      dwv[v] = dwv[v] + f * d;
    }
  }
  if (A.forcing) {  // euler.f90:294-318
#pragma unroll
    for (int v = 0; v < 5; v++) {
      T q;
      if (A.first_forcing) {
        q = T(0);
        if (b.marker[c] == 1) q = T(1) * b.wr[v * N + c] - dwv[v];
        b.qf[v * N + c] = q;
      } else {
        q = b.qf[v * N + c];
      }
      dwv[v] = dwv[v] + q;
    }
    if (P.unsteady) {
      const T lam = unsteady_lam(b, P, A, c), rl = T(1) / lam;
#pragma unroll
      for (int v = 0; v < 5; v++) dwv[v] = mdiv(dwv[v], lam, rl);
    }
  }
  if (FAST) {
    if (b.blank[c] == 0)
#pragma unroll
      for (int v = 0; v < 5; v++) dwv[v] = T(0);
  } else if (b.blank[c] == 0) {
    // dw * blank: x * 1 is x itself, so only blanked cells multiply (by 0)
#pragma unroll
    for (int v = 0; v < 5; v++) dwv[v] = dwv[v] * T(0);
  }
  if (A.lres) {
#pragma unroll
    for (int v = 0; v < 5; v++) b.dw[v * N + c] = dwv[v];
    return;
  }
  // time-step scaling, euler.f90:364-372: de = fn*vdtim/cellvolume
  T vd = A.vt ? (T)(*b.dtim) : b.vdtim[c];
  T de = FAST ? ((T)A.fn * vd) * rcp_vol(b) : smdiv(smul((T)A.fn, vd), (T)b.vol, rcp_vol(b));
#pragma unroll
  for (int v = 0; v < 5; v++) dwv[v] = smul(de, dwv[v]);
  if (A.irs) {
#pragma unroll
    for (int v = 0; v < 5; v++) b.dw[v * N + c] = dwv[v];
    return;
  }
  // update, euler.f90:381-399 (steady: lam = 1, and dw/1 is dw)
  T wv[5];
  if (P.unsteady && !A.forcing) {
    const T lam = unsteady_lam(b, P, A, c), rl = T(1) / lam;
#pragma unroll
    for (int v = 0; v < 5; v++) wv[v] = b.wn[v * N + c] - mdiv(dwv[v], lam, rl);
  } else {
#pragma unroll
    for (int v = 0; v < 5; v++) wv[v] = b.wn[v * N + c] - dwv[v];
  }
#pragma unroll
  for (int v = 0; v < 5; v++) {
    b.w[v * N + c] = wv[v];
    b.dw[v * N + c] = dwv[v];
  }
  b.p[c] = depvars((T)P.gamma, wv);
}

// --------------------------------------------------------------- implicit residual smoothing
// psmoo_old (psmoo.f90:97-242): constant-coefficient Thomas sweeps along i,
// then j, then k, skipping blanked cells without re-factoring the pivots.
// One thread per (line, variable); consecutive threads walk consecutive
// lines of one variable, so the j- and k-sweeps are coalesced.  TC is the
// arithmetic precision.
template <typename T, int D>
__device__ __forceinline__ long long irs_lines(const DevBlock<T>& b) {
  return D == 0 ? (long long)b.ny * b.nz : (D == 1 ? (long long)b.nx * b.nz : (long long)b.nx * b.ny);
}

// SC: the products of the forward and backward steps on the integer pipes.
// That lengthens the serial chain of each line, so it pays only where many
// lines run at once and the sweep is bound by the FP64 rate; with few lines
// (coarse levels, slabs) the chain's latency bounds it and the FP64 forms
// are faster.
template <typename T, typename TC, int D, bool SC = false>
__device__ __forceinline__ void body_irs(const DevBlock<T>& b, const IrsTables& tb, TC bb, long long t) {
  const long long lines = irs_lines<T, D>(b);
  const int v = (int)(t / lines);
  const long long ln = t - (long long)v * lines;
  long long c0, st;
  int l;
  if (D == 0) {
    int j = 2 + (int)(ln % b.ny), k = 2 + (int)(ln / b.ny);
    c0 = cidx(b.Pi, b.Pj, 0, j, k);
    st = 1;
    l = b.il;
  } else if (D == 1) {
    int i = 2 + (int)(ln % b.nx), k = 2 + (int)(ln / b.nx);
    c0 = cidx(b.Pi, b.Pj, i, 0, k);
    st = b.Pi;
    l = b.jl;
  } else {
    int i = 2 + (int)(ln % b.nx), j = 2 + (int)(ln / b.nx);
    c0 = cidx(b.Pi, b.Pj, i, j, 0);
    st = (long long)b.Pi * b.Pj;
    l = b.kl;
  }
  T* d = b.dw + (long long)v * b.N;
  TC prev;
  {
    long long c = c0 + 2 * st;
    TC x = (TC)d[c];
    if (b.blank[c] != 0) {
      x = x / irs_e1(tb, 2, TC(0));
      d[c] = (T)x;
    }
    prev = x;
  }
  // The recurrence is serial, its loads are not: each chunk of K cells is
  // loaded before any of it is solved, so one memory latency is paid per
  // chunk instead of per cell.  Every cell is read once and written once
  // after its own read, so the order of results is unchanged.
  constexpr int K = 8;
  TC xb[K], pb[K], rb[K];
  unsigned char bk[K];
  for (int q0 = 3; q0 <= l; q0 += K) {
#pragma unroll
    for (int u = 0; u < K; u++)
      if (q0 + u <= l) {
        const long long c = c0 + (q0 + u) * st;
        xb[u] = (TC)d[c];
        bk[u] = b.blank[c];
        pb[u] = irs_e1(tb, q0 + u, TC(0));
        rb[u] = irs_e1r(tb, q0 + u, TC(0));
      }
#pragma unroll
    for (int u = 0; u < K; u++)
      if (q0 + u <= l) {
        TC x = xb[u];
        if (bk[u] != 0) {
          x = SC ? smdiv(x - smul(bb, prev), pb[u], rb[u]) : mdiv(x - bb * prev, pb[u], rb[u]);
          d[c0 + (q0 + u) * st] = (T)x;
        }
        prev = x;
      }
  }
  for (int q0 = l - 1; q0 >= 2; q0 -= K) {
#pragma unroll
    for (int u = 0; u < K; u++)
      if (q0 - u >= 2) {
        const long long c = c0 + (q0 - u) * st;
        xb[u] = (TC)d[c];
        bk[u] = b.blank[c];
        pb[u] = irs_e2(tb, q0 - u, TC(0));
      }
#pragma unroll
    for (int u = 0; u < K; u++)
      if (q0 - u >= 2) {
        TC x = xb[u];
        if (bk[u] != 0) {
          x = x - (SC ? smul(pb[u], prev) : pb[u] * prev);
          d[c0 + (q0 - u) * st] = (T)x;
        }
        prev = x;
      }
  }
}

// The FP32 sweeps of the mixed form's finest level, whose storage is FP64.
// body_irs<double, float, D> converts every value on its way in and out of
// each sweep, and on this part those conversions issue at the FP64 rate.
// Here the i sweep reads dw and leaves its results in an FP32 copy (in the
// stage scratch, free after the residual pass); the j sweep works in the
// copy; the k sweep writes its results back to dw.  A float stored as double
// and read back is the same float, so every value is the one body_irs gives;
// blanked cells keep their dw, as there.
template <typename TS, typename TO, int D>
__device__ __forceinline__ void body_irs_mixed(const DevBlock<double>& b, const IrsTables& tb, float bb,
                                               const TS* src, float* mid, TO* out, long long t) {
  constexpr bool fill = !std::is_same<TS, float>::value;  // the i sweep: every cell into the copy
  constexpr bool back = !std::is_same<TO, float>::value;  // the k sweep: results back to dw
  const long long lines = irs_lines<double, D>(b);
  const int v = (int)(t / lines);
  const long long ln = t - (long long)v * lines;
  long long c0, st;
  int l;
  if (D == 0) {
    int j = 2 + (int)(ln % b.ny), k = 2 + (int)(ln / b.ny);
    c0 = cidx(b.Pi, b.Pj, 0, j, k);
    st = 1;
    l = b.il;
  } else if (D == 1) {
    int i = 2 + (int)(ln % b.nx), k = 2 + (int)(ln / b.nx);
    c0 = cidx(b.Pi, b.Pj, i, 0, k);
    st = b.Pi;
    l = b.jl;
  } else {
    int i = 2 + (int)(ln % b.nx), j = 2 + (int)(ln / b.nx);
    c0 = cidx(b.Pi, b.Pj, i, j, 0);
    st = (long long)b.Pi * b.Pj;
    l = b.kl;
  }
  const TS* s = src + (long long)v * b.N;
  float* m = mid + (long long)v * b.N;
  TO* o = out + (long long)v * b.N;
  float prev;
  {
    const long long c = c0 + 2 * st;
    float x = (float)s[c];
    if (b.blank[c] != 0) {
      x = x / irs_e1(tb, 2, 0.0f);
      m[c] = x;
    } else if (fill) {
      m[c] = x;
    }
    prev = x;
  }
  constexpr int K = 8;
  float xb[K], pb[K], rb[K];
  unsigned char bk[K];
  for (int q0 = 3; q0 <= l; q0 += K) {
#pragma unroll
    for (int u = 0; u < K; u++)
      if (q0 + u <= l) {
        const long long c = c0 + (q0 + u) * st;
        xb[u] = (float)s[c];
        bk[u] = b.blank[c];
        pb[u] = irs_e1(tb, q0 + u, 0.0f);
        rb[u] = irs_e1r(tb, q0 + u, 0.0f);
      }
#pragma unroll
    for (int u = 0; u < K; u++)
      if (q0 + u <= l) {
        float x = xb[u];
        if (bk[u] != 0) {
          x = mdiv(x - bb * prev, pb[u], rb[u]);
          m[c0 + (q0 + u) * st] = x;
        } else if (fill) {
          m[c0 + (q0 + u) * st] = x;
        }
        prev = x;
      }
  }
  // the backward pass does not revisit row l: its forward result is final
  if (back && b.blank[c0 + l * st] != 0) o[c0 + l * st] = (TO)prev;
  for (int q0 = l - 1; q0 >= 2; q0 -= K) {
#pragma unroll
    for (int u = 0; u < K; u++)
      if (q0 - u >= 2) {
        const long long c = c0 + (q0 - u) * st;
        xb[u] = m[c];
        bk[u] = b.blank[c];
        pb[u] = irs_e2(tb, q0 - u, 0.0f);
      }
#pragma unroll
    for (int u = 0; u < K; u++)
      if (q0 - u >= 2) {
        float x = xb[u];
        if (bk[u] != 0) {
          x = x - pb[u] * prev;
          o[c0 + (q0 - u) * st] = (TO)x;
        }
        prev = x;
      }
  }
}

// The mixed form's i sweep with one warp per (line, variable).  A psmoo_old
// row is an affine map of the row before it, x(q) = a(q) x(q-1) + c(q):
// forward a = -bb/e1(q), c = dw(q)/e1(q) on unblanked rows and a = 0,
// c = dw(q) on blanked ones (the row keeps its value, and the next row
// takes it as its predecessor); backward a = -e2(q), c = x(q) on unblanked
// rows.  Each lane composes the maps of K consecutive rows, a warp scan of
// the composed maps gives every lane the value entering its rows, and the
// lane applies its maps in order.  Loads and stores of a warp cover one
// contiguous line.  FP32 arithmetic: on the FP64 residual of the mixed
// form's finest level, the result going to the FP32 copy the j and k sweeps
// continue on; or on an FP32 level's residual, in place (every row of the
// line, blanked rows with their unsmoothed value).
template <int K, typename T = double>
__global__ void __launch_bounds__(256) k_irs_scan_i(DevBlock<T> b, IrsTables tb, float bb, float* cp) {
  const long long lines = (long long)b.ny * b.nz;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wid >= 5 * lines) return;  // uniform over the warp
  const int v = (int)(wid / lines);
  const long long ln = wid - (long long)v * lines;
  const int j = 2 + (int)(ln % b.ny), k = 2 + (int)(ln / b.ny);
  const long long c0 = cidx(b.Pi, b.Pj, 0, j, k);
  const int l = b.il;
  const T* src = b.dw + (long long)v * b.N + c0;  // read whole into registers before any write
  float* dst = cp + (long long)v * b.N + c0;
  const uint8_t* bl = b.blank + c0;
  const int q0 = 2 + lane * K;
  float x[K];
  unsigned bk = 0;
  // forward: the lane's maps, composed in row order
  float ca = 1.f, cc = 0.f;
#pragma unroll
  for (int u = 0; u < K; u++) {
    const int q = q0 + u;
    if (q <= l) {
      const float d = (float)src[q];
      float a = 0.f, c = d;
      if (bl[q] != 0) {
        bk |= 1u << u;
        const float r = irs_e1r(tb, q, 0.0f);
        a = q == 2 ? 0.f : -bb * r;
        c = d * r;
      }
      x[u] = c;
      ca = a * ca;
      cc = fmaf(a, cc, c);
    } else {
      x[u] = 0.f;
    }
  }
  // inclusive scan over the lanes in row order, then the value entering
  // this lane's first row (row 2's map ignores its input: a = 0)
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const float pa = __shfl_up_sync(0xffffffffu, ca, off), pc = __shfl_up_sync(0xffffffffu, cc, off);
    if (lane >= off) {
      cc = fmaf(ca, pc, cc);
      ca = ca * pa;
    }
  }
  float prev = __shfl_up_sync(0xffffffffu, cc, 1);
  if (lane == 0) prev = 0.f;
#pragma unroll
  for (int u = 0; u < K; u++) {
    const int q = q0 + u;
    if (q <= l && q > 2 && (bk >> u & 1u)) x[u] = fmaf(-bb * irs_e1r(tb, q, 0.0f), prev, x[u]);
    if (q <= l) prev = x[u];
  }
  // backward: rows l-1 down to 2; row l keeps its forward value
  ca = 1.f;
  cc = 0.f;
#pragma unroll
  for (int u = K - 1; u >= 0; u--) {
    const int q = q0 + u;
    if (q <= l) {
      const float a = (q < l && (bk >> u & 1u)) ? -irs_e2(tb, q, 0.0f) : 0.f;
      ca = a * ca;
      cc = fmaf(a, cc, x[u]);
    }
  }
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const float pa = __shfl_down_sync(0xffffffffu, ca, off), pc = __shfl_down_sync(0xffffffffu, cc, off);
    if (lane + off < 32) {
      cc = fmaf(ca, pc, cc);
      ca = ca * pa;
    }
  }
  prev = __shfl_down_sync(0xffffffffu, cc, 1);
  if (lane == 31) prev = 0.f;
#pragma unroll
  for (int u = K - 1; u >= 0; u--) {
    const int q = q0 + u;
    if (q <= l) {
      if (q < l && (bk >> u & 1u)) x[u] = fmaf(-irs_e2(tb, q, 0.0f), prev, x[u]);
      prev = x[u];
      dst[q] = x[u];
    }
  }
}

// the rows a lane of k_irs_scan_i takes for a line of len rows (0: none fits)
inline int irs_scan_k(int len) {
  const int need = (len + 31) / 32;
  const int ks[] = {2, 4, 6, 8, 12, 16};
  for (int q : ks)
    if (need <= q) return q;
  return 0;
}

template <typename TS, typename TO, int D>
__global__ void k_irs_mixed(DevBlock<double> b, IrsTables tb, float bb, const TS* src, float* mid, TO* out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < 5 * irs_lines<double, D>(b)) body_irs_mixed<TS, TO, D>(b, tb, bb, src, mid, out, t);
}

// Shared-memory variant of body_irs: a block stages LT whole lines of one
// variable (and their blanking) in shared memory with coalesced loads, each
// of its first LT threads runs the reference's sweep on one line there, and
// the block writes the lines back coalesced.  Arithmetic and order per line
// are those of body_irs.
// Loads from src and stores to dst (both dw, except for the FP32 copy of the
// mixed form's i sweep: dw in, the copy out, every cell of the tile written)
template <typename T, typename TC, int D, int LT, typename TS, typename TO>
__device__ __forceinline__ void body_irs_smem(const DevBlock<T>& b, const IrsTables& tb, TC bb, const TS* src,
                                              TO* dst) {
  extern __shared__ unsigned char smem_raw[];
  const long long lines = irs_lines<T, D>(b);
  const long long ntile = (lines + LT - 1) / LT;
  const int v = (int)(blockIdx.x / ntile);
  const long long tile = blockIdx.x - (long long)v * ntile;
  const long long l0 = tile * LT;
  const int nl = (int)min((long long)LT, lines - l0);
  const int l = (D == 0) ? b.il : (D == 1 ? b.jl : b.kl);   // rows 2..l
  const int len = l - 1;
  const int S = (D == 0) ? (len | 1) : LT;                  // odd row stride for line-major tiles
  TC* x = (TC*)smem_raw;
  unsigned char* bl = smem_raw + sizeof(TC) * (size_t)LT * (len + 1);
  const TS* d = src + (long long)v * b.N;
  TO* dout = dst + (long long)v * b.N;
  const long long N = b.N;
  (void)N;
  // element (line r, row q) of the tile -> global cell
  auto cell = [&](int r, int q) -> long long {
    long long ln = l0 + r;
    if (D == 0) {
      int j = 2 + (int)(ln % b.ny), k = 2 + (int)(ln / b.ny);
      return cidx(b.Pi, b.Pj, 2 + q, j, k);
    } else if (D == 1) {
      int i = 2 + (int)(ln % b.nx), k = 2 + (int)(ln / b.nx);
      return cidx(b.Pi, b.Pj, i, 2 + q, k);
    } else {
      int i = 2 + (int)(ln % b.nx), j = 2 + (int)(ln / b.nx);
      return cidx(b.Pi, b.Pj, i, j, 2 + q);
    }
  };
  auto sidx = [&](int r, int q) -> int { return D == 0 ? r * S + q : q * LT + r; };
  const int tot = nl * len;
  for (int e = threadIdx.x; e < LT * len; e += blockDim.x) {
    int r, q;
    if (D == 0) { r = e / len; q = e - r * len; } else { q = e / LT; r = e - q * LT; }
    if (r < nl) {
      long long c = cell(r, q);
      x[sidx(r, q)] = (TC)d[c];
      bl[sidx(r, q)] = b.blank[c];
    }
  }
  __syncthreads();
  const int r = threadIdx.x;
  if (r < nl) {
    TC prev;
    {
      TC xv = x[sidx(r, 0)];
      if (bl[sidx(r, 0)] != 0) {
        xv = xv / irs_e1(tb, 2, TC(0));
        x[sidx(r, 0)] = xv;
      }
      prev = xv;
    }
    for (int q = 1; q < len; q++) {
      TC xv = x[sidx(r, q)];
      if (bl[sidx(r, q)] != 0) {
        xv = mdiv(xv - bb * prev, irs_e1(tb, q + 2, TC(0)), irs_e1r(tb, q + 2, TC(0)));
        x[sidx(r, q)] = xv;
      }
      prev = xv;
    }
    for (int q = len - 2; q >= 0; q--) {
      TC xv = x[sidx(r, q)];
      if (bl[sidx(r, q)] != 0) {
        xv = xv - irs_e2(tb, q + 2, TC(0)) * prev;
        x[sidx(r, q)] = xv;
      }
      prev = xv;
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < LT * len; e += blockDim.x) {
    int rr, q;
    if (D == 0) { rr = e / len; q = e - rr * len; } else { q = e / LT; rr = e - q * LT; }
    if (rr < nl) dout[cell(rr, q)] = (TO)x[sidx(rr, q)];
  }
  (void)tot;
}

template <typename T, typename TC, int D, int LT>
__global__ void __launch_bounds__(LT) k_irs_smem(DevBlock<T> b, IrsTables tb, TC bb) {
  body_irs_smem<T, TC, D, LT>(b, tb, bb, (const T*)b.dw, b.dw);
}

// the mixed form's i sweep in shared-memory tiles: dw in, the FP32 copy out
template <int LT>
__global__ void __launch_bounds__(LT) k_irs_smem_fill(DevBlock<double> b, IrsTables tb, float bb, float* cp) {
  body_irs_smem<double, float, 0, LT>(b, tb, bb, (const double*)b.dw, cp);
}

template <typename TC, int LT>
size_t irs_smem_bytes(int len) {
  return sizeof(TC) * (size_t)LT * (len + 1) + (size_t)LT * (len + 1);
}

// update after smoothing, euler.f90:381-399 (steady: lam = 1)
// --------------------------------------------------------------- psmoo + progon3 (irs_variant 1)
// psmoo.f90:1-95 with progon3.f90:41-60: per-cell coefficients eps from the
// time step, aa = 1+2eps, bb = cc = -eps with the end couplings zeroed
// (psmoo.f90:49-50), solved by progon3's forward/backward recurrences.  One
// thread per line carries all five variables: the coefficient recurrences v
// and w do not depend on the variable and are formed once.  The recurrences
// pass through the stage scratch F, dead between the residual pass and the
// next stage: slot q of a line holds progon3's v(q), w(q), u(q,1:5) on the
// way forward and s(q-1), t(q-1,1:5) on the way back.
template <typename T, int D>
__device__ __forceinline__ void line_of(const DevBlock<T>& b, long long ln, long long& c0, long long& st, int& l) {
  if (D == 0) {
    int j = 2 + (int)(ln % b.ny), k = 2 + (int)(ln / b.ny);
    c0 = cidx(b.Pi, b.Pj, 0, j, k);
    st = 1;
    l = b.il;
  } else if (D == 1) {
    int i = 2 + (int)(ln % b.nx), k = 2 + (int)(ln / b.nx);
    c0 = cidx(b.Pi, b.Pj, i, 0, k);
    st = b.Pi;
    l = b.jl;
  } else {
    int i = 2 + (int)(ln % b.nx), j = 2 + (int)(ln / b.nx);
    c0 = cidx(b.Pi, b.Pj, i, j, 0);
    st = (long long)b.Pi * b.Pj;
    l = b.kl;
  }
}

template <typename T, typename TC, int D>
__device__ __noinline__ void body_psmoo_line(const DevBlock<T>& b, long long ln) {
  const long long N = b.N;
  long long c0, st;
  int l;
  line_of<T, D>(b, ln, c0, st, l);
  const T* eps = b.eps + (long long)D * N;
  T* Sv = b.F;          // v forward, s backward
  T* Sw = b.F + N;      // w forward
  T* Su = b.F + 2 * N;  // u(1:5) forward, t(1:5) backward
  // forward: equation i = 1..n sits at cell q = i+1 = 2..l (n = l-1)
  TC v = TC(0), w = TC(1), u[5];
#pragma unroll
  for (int x = 0; x < 5; x++) u[x] = TC(0);
  for (int q = 2; q <= l; q++) {
    const long long c = c0 + q * st;
    const TC e = (TC)eps[c];
    const TC a = TC(1) + TC(2) * e;
    const TC bq = (q == l) ? TC(0) : -e;
    const TC cq = (q == 2) ? TC(0) : -e;
    const TC z = TC(1) / (a + cq * v);
    v = -bq * z;
#pragma unroll
    for (int x = 0; x < 5; x++) u[x] = (-cq * u[x] + (TC)b.dw[x * N + c]) * z;
    w = -cq * w * z;
    if (q < l) {  // v(n+1), w(n+1), u(n+1) are never read back
      Sv[c] = (T)v;
      Sw[c] = (T)w;
#pragma unroll
      for (int x = 0; x < 5; x++) Su[x * N + c] = (T)u[x];
    }
  }
  // backward: s(i) = v(i+1) s(i+1) + w(i+1), t likewise, i = n-1..1, read
  // from slot i+1 and stored back there; s(n-1), t(n-1) are kept for x(n)
  // (zero when n = 1, progon3's s(0), t(0))
  TC s = TC(1), t[5], shi = TC(0), thi[5];
#pragma unroll
  for (int x = 0; x < 5; x++) t[x] = thi[x] = TC(0);
  for (int q = l - 1; q >= 2; q--) {
    const long long c = c0 + q * st;
    const TC vv = (TC)Sv[c], ww = (TC)Sw[c];
    s = vv * s + ww;
#pragma unroll
    for (int x = 0; x < 5; x++) t[x] = vv * t[x] + (TC)Su[x * N + c];
    Sv[c] = (T)s;
#pragma unroll
    for (int x = 0; x < 5; x++) Su[x * N + c] = (T)t[x];
    if (q == l - 1) {
      shi = s;
#pragma unroll
      for (int x = 0; x < 5; x++) thi[x] = t[x];
    }
  }
  // x(n) at cell l, then x(i) = s(i) x(n) + t(i) at cells 2..l-1
  const long long cl = c0 + l * st;
  const TC el = (TC)eps[cl];
  const TC an = TC(1) + TC(2) * el, bn = TC(0), cn = (l == 2) ? TC(0) : -el;
  const TC den = an + bn * s + cn * shi;
  TC xn[5];
#pragma unroll
  for (int x = 0; x < 5; x++) xn[x] = ((TC)b.dw[x * N + cl] - bn * t[x] - cn * thi[x]) / den;
  for (int q = 2; q <= l - 1; q++) {
    const long long c = c0 + q * st;
    const TC sv = (TC)Sv[c];
#pragma unroll
    for (int x = 0; x < 5; x++) b.dw[x * N + c] = (T)(sv * xn[x] + (TC)Su[x * N + c]);
  }
#pragma unroll
  for (int x = 0; x < 5; x++) b.dw[x * N + cl] = (T)xn[x];
}

template <typename T, typename TC, int D>
__global__ void k_psmoo_line(DevBlock<T> b) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < irs_lines<T, D>(b)) body_psmoo_line<T, TC, D>(b, t);
}

template <typename T>
__device__ __forceinline__ void body_update(const DevBlock<T>& b, const PhysParams& P, const StageArgs& A,
                                            long long t) {
  int i = 2 + (int)(t % b.nx);
  int j = 2 + (int)((t / b.nx) % b.ny);
  int k = 2 + (int)(t / ((long long)b.nx * b.ny));
  const long long N = b.N;
  const long long c = cidx(b.Pi, b.Pj, i, j, k);
  T wv[5];
  if (P.unsteady && !A.forcing) {
    const T lam = unsteady_lam(b, P, A, c), rl = T(1) / lam;
#pragma unroll
    for (int v = 0; v < 5; v++) wv[v] = b.wn[v * N + c] - mdiv(b.dw[v * N + c], lam, rl);
  } else {
#pragma unroll
    for (int v = 0; v < 5; v++) wv[v] = b.wn[v * N + c] - b.dw[v * N + c];
  }
#pragma unroll
  for (int v = 0; v < 5; v++) b.w[v * N + c] = wv[v];
  b.p[c] = depvars((T)P.gamma, wv);
}

// --------------------------------------------------------------- bc_cutcell (bc_cutcell.f90:40-268)
template <typename T>
__device__ void body_cutcell(const DevBlock<T>& b, const PhysParams& P, unsigned* err, int m) {
  if (m >= b.nmir || m > b.m0) return;
  T* ws = b.rec_wsol + 5LL * m;
  if (m == b.m0) {  // empty cloud: zero this record; the reference returns here
    for (int v = 0; v < 5; v++) ws[v] = T(0);
    b.rec_psol[m] = T(0);
    return;
  }
  const long long N = b.N;
  const int ncl = b.rec_i[8 * m + 5];
  T nv[3] = {(T)b.rec_nvec[3 * m], (T)b.rec_nvec[3 * m + 1], (T)b.rec_nvec[3 * m + 2]};
  T qb[3] = {(T)b.rec_qb[3 * m], (T)b.rec_qb[3 * m + 1], (T)b.rec_qb[3 * m + 2]};
  T nn = sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
  for (int q = 0; q < 3; q++) nv[q] = nv[q] / nn;
  long long cl[8];
  T cf[8];
  for (int q = 0; q < ncl; q++) {
    const int* ijk = b.rec_cloud + (8 * m + q) * 3;
    cl[q] = cidx(b.Pi, b.Pj, ijk[0], ijk[1], ijk[2]);
    cf[q] = (T)b.rec_coef[8 * m + q];
  }
  T vr[5];
  for (int v = 0; v < 5; v++) {
    T a = T(0);
    for (int q = 0; q < ncl; q++) a = a + cf[q] * b.w[v * N + cl[q]];
    vr[v] = a;
  }
  T pr = T(0);
  for (int q = 0; q < ncl; q++) pr = pr + cf[q] * b.p[cl[q]];
  T wsol[5], psol = pr;
  const T gm1 = (T)P.gamma - T(1);
  if (!P.eqn_ns) {
    for (int v = 0; v < 5; v++) wsol[v] = vr[v];
    T qn = T(2) * (nv[0] * (wsol[1] - wsol[0] * qb[0]) + nv[1] * (wsol[2] - wsol[0] * qb[1]) +
                   nv[2] * (wsol[3] - wsol[0] * qb[2]));
    for (int q = 0; q < 3; q++) wsol[1 + q] = wsol[1 + q] - qn * nv[q];
  } else {
    wsol[0] = vr[0];
    for (int q = 0; q < 3; q++) wsol[1 + q] = T(2) * qb[q] * vr[0] - vr[1 + q];
  }
  wsol[4] = psol / gm1 + T(0.5) * (wsol[1] * wsol[1] + wsol[2] * wsol[2] + wsol[3] * wsol[3]) / wsol[0];
  bool nan = false;
  for (int v = 0; v < 5; v++) nan |= (wsol[v] != wsol[v]);
  if (nan && !P.eqn_ns) atomicCAS(err, 0u, (unsigned)ERR_NAN);
  for (int v = 0; v < 5; v++) ws[v] = wsol[v];
  b.rec_psol[m] = psol;
}

// --------------------------------------------------------------- face boundary conditions
// One launch per face in the order 1..6 of bcond.f90:16-39: later faces read
// and overwrite ghost cells that earlier faces wrote.
// the far field's powers: the short forms for gamma = 1.4 in FP64 (fast_pow.cuh)
__device__ __forceinline__ double pow_gm(const PhysParams& P, double x, double gm) {
  if (P.gamma14) return pow_5_2(x, P.pow_dm);
  return pow(x, gm);
}
__device__ __forceinline__ float pow_gm(const PhysParams&, float x, float gm) { return pow(x, gm); }
__device__ __forceinline__ double pow_gamma(const PhysParams& P, double x, double gamma) {
  if (P.gamma14) return pow_7_5(x, P.pow_dg);
  return pow(x, gamma);
}
__device__ __forceinline__ float pow_gamma(const PhysParams&, float x, float gamma) { return pow(x, gamma); }

template <typename T>
__device__ void body_bc_face(const DevBlock<T>& b, const PhysParams& P, int face, long long t) {
  const int ax = (face - 1) % 3;
  const int na = (ax == 0 ? b.jb : b.ib) + 1;  // first tangential extent
  int t1 = (int)(t % na), t2 = (int)(t / na);
  const int kind = b.bctype[face - 1];
  const int lcur = ax == 0 ? b.il : (ax == 1 ? b.jl : b.kl);
  auto at = [&](int q) -> long long {
    if (ax == 0) return cidx(b.Pi, b.Pj, q, t1, t2);
    if (ax == 1) return cidx(b.Pi, b.Pj, t1, q, t2);
    return cidx(b.Pi, b.Pj, t1, t2, q);
  };
  const long long N = b.N;
  int phy1, phy2, dum1, dum2;
  if (kind == -60) {
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
  const long long d1 = at(dum1), d2 = at(dum2), p1 = at(phy1), p2 = at(phy2);
  if (kind == -20) {  // bc_far.f90:42-284
    const T gamma = (T)P.gamma, gm = (T)P.gm;
    const T fn0 = (T)b.fnv[face - 1][0], fn1 = (T)b.fnv[face - 1][1], fn2 = (T)b.fnv[face - 1][2];
    const T fnn = (T)b.fnv[face - 1][ax];
    T wp[5];
    for (int v = 0; v < 5; v++) wp[v] = b.w[v * N + p1];
    T pph = b.p[p1];
    // the quotients by the cell's density share one reciprocal, those by
    // gamma-1 and gamma take the host's (mdiv: the same roundings as the
    // divisions, with a shorter dependent chain)
    const T y0 = T(1) / wp[0], gm1 = gamma - T(1), rg1 = rcp_gm1(P, T(0)), rgam = rcp_gamma(P, T(0));
    T vel_norm = mdiv(wp[1] * fn0 + wp[2] * fn1 + wp[3] * fn2, wp[0], y0);
    T out[5], pout;
    bool set = false;
    const T u0a = (T)P.u0[ax];
    const T rmi = u0a * fnn - mdiv(T(2) * (T)P.c0, gm1, rg1);
    if (vel_norm <= T(0)) {
      T rhoe = wp[0];
      T ue = mdiv(wp[1 + ax], rhoe, y0);
      T pe = pph;
      T ce = sqrt(mdiv(gamma * pe, rhoe, y0));
      T rpo = ue * fnn + mdiv(T(2) * ce, gm1, rg1);
      T vv[3] = {(T)P.u0[0], (T)P.u0[1], (T)P.u0[2]};
      vv[ax] = T(0.5) * (rpo + rmi) * fnn;
      T ci = T(0.25) * (gamma - T(1)) * (rpo - rmi);
      T si = (T)P.si_far;
      T cc = mdiv(ci * ci, gamma, rgam);
      T rhoi = pow_gm(P, si * cc, gm);
      T prei = rhoi * cc;
      out[0] = rhoi;
      out[1] = rhoi * vv[0];
      out[2] = rhoi * vv[1];
      out[3] = rhoi * vv[2];
      out[4] = prei * gm + T(0.5) * rhoi * (vv[0] * vv[0] + vv[1] * vv[1] + vv[2] * vv[2]);
      pout = prei;
      set = true;
    } else if (vel_norm > T(0)) {
      T rhoi = wp[0];
      T vv[3] = {mdiv(wp[1], rhoi, y0), mdiv(wp[2], rhoi, y0), mdiv(wp[3], rhoi, y0)};
      T prei = pph;
      T si = pow_gamma(P, rhoi, gamma) / prei;
      T ci = sqrt(mdiv(gamma * prei, rhoi, y0));
      T rpo = vv[ax] * fnn + mdiv(T(2) * ci, gm1, rg1);
      T ve[3] = {vv[0], vv[1], vv[2]};
      ve[ax] = T(0.5) * (rpo + rmi) * fnn;
      T ce = T(0.25) * (gamma - T(1)) * (rpo - rmi);
      T cc = mdiv(ce * ce, gamma, rgam);
      T rhoe = pow_gm(P, si * cc, gm);
      T pe = rhoe * cc;
      out[0] = rhoe;
      out[1] = rhoe * ve[0];
      out[2] = rhoe * ve[1];
      out[3] = rhoe * ve[2];
      out[4] = pe * gm + T(0.5) * rhoe * (ve[0] * ve[0] + ve[1] * ve[1] + ve[2] * ve[2]);
      pout = pe;
      set = true;
    }
    if (set) {  // both ghost layers take the new state
      for (int v = 0; v < 5; v++) {
        b.w[v * N + d1] = out[v];
        b.w[v * N + d2] = out[v];
      }
      b.p[d1] = pout;
      b.p[d2] = pout;
    } else {  // vel_norm NaN: the second layer copies the first as it stands
      for (int v = 0; v < 5; v++) b.w[v * N + d2] = b.w[v * N + d1];
      b.p[d2] = b.p[d1];
    }
  } else if (kind == -50) {  // bc_symm.f90
    for (int v = 0; v < 5; v++) b.w[v * N + d1] = b.w[v * N + p1];
    b.w[(1 + ax) * N + d1] = -b.w[(1 + ax) * N + p1];
    b.p[d1] = b.p[p1];
    for (int v = 0; v < 5; v++) b.w[v * N + d2] = b.w[v * N + p2];
    b.w[(1 + ax) * N + d2] = -b.w[(1 + ax) * N + p2];
    b.p[d2] = b.p[p2];
  } else if (kind == -80) {  // bc_wall.f90
    b.w[d1] = b.w[p1];
    b.w[4 * N + d1] = b.w[4 * N + p1];
    for (int v = 1; v < 4; v++) b.w[v * N + d1] = -b.w[v * N + p1];
    b.w[d2] = b.w[p2];
    b.w[4 * N + d2] = b.w[4 * N + p2];
    for (int v = 1; v < 4; v++) b.w[v * N + d2] = -b.w[v * N + p2];
    b.p[d1] = b.p[p1];
    b.p[d2] = b.p[p1];
  } else if (kind == -60) {  // bc_periodic.f90
    for (int v = 0; v < 5; v++) b.w[v * N + d2] = b.w[v * N + p2];
    for (int v = 0; v < 5; v++) b.w[v * N + d1] = b.w[v * N + p1];
    b.p[d2] = b.p[p2];
    b.p[d1] = b.p[p1];
  }
}

// bcond.f90:16-42 applies the faces 1..6 one after the other over their
// whole tangential range, so a later face overwrites the edge and corner
// ghosts of an earlier one and reads what the earlier one wrote.  The same
// result comes from three passes over all faces at once, by the number of
// ghost coordinates among a ghost cell's two tangential ones (0: face
// ghosts, 1: edges, 2: corners), each cell written only by its last writer,
// the highest-numbered face (with a boundary condition) whose axis is a
// ghost axis of the cell.  That writer reads cells with one ghost axis fewer,
// whose own writers all come before it, so every read sees the value the
// sequential order leaves there.
template <typename T>
__device__ __forceinline__ long long bc_pass_items(const DevBlock<T>& b) {
  const long long s0 = (long long)(b.jb + 1) * (b.kb + 1), s1 = (long long)(b.ib + 1) * (b.kb + 1),
                  s2 = (long long)(b.ib + 1) * (b.jb + 1);
  return 2 * (s0 + s1 + s2);
}

template <typename T>
__device__ __forceinline__ void body_bc_pass(const DevBlock<T>& b, const PhysParams& P, int pass, long long t) {
  const long long sz[3] = {(long long)(b.jb + 1) * (b.kb + 1), (long long)(b.ib + 1) * (b.kb + 1),
                           (long long)(b.ib + 1) * (b.jb + 1)};
  int face = 1;
  while (face < 6 && t >= sz[(face - 1) % 3]) {
    t -= sz[(face - 1) % 3];
    face++;
  }
  if (b.bctype[face - 1] == 0) return;
  const int ax = (face - 1) % 3;
  const int na = (ax == 0 ? b.jb : b.ib) + 1;
  const int t1 = (int)(t % na), t2 = (int)(t / na);
  const int ta = ax == 0 ? 1 : 0, tb = ax == 2 ? 1 : 2;  // tangential axes of t1, t2
  const int lim[3] = {b.il, b.jl, b.kl};
  int deg = 0;
  bool last = true;
  auto tangential = [&](int a, int q) {
    const int g = q <= 1 ? a + 1 : (q > lim[a] ? a + 4 : 0);  // the face whose ghosts hold q
    if (g) {
      deg++;
      if (g > face && b.bctype[g - 1] != 0) last = false;
    }
  };
  tangential(ta, t1);
  tangential(tb, t2);
  if (deg == pass && last) body_bc_face(b, P, face, t);
}

template <typename T>
__global__ void k_bc_pass(DevBlock<T> b, PhysParams P, int pass) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < bc_pass_items(b)) body_bc_pass(b, P, pass, t);
}

// bc_corner.f90:23-157: three dependent phases, each a set of independent
// items (phase 0: edges along k and j, phase 1: edges along i, phase 2: the
// eight corners); no item of a phase reads a cell another item of the same
// phase writes
template <typename T>
__device__ __forceinline__ int corner_items(const DevBlock<T>& b, int phase) {
  return phase == 0 ? 4 * (b.kl - 1) + 4 * (b.jl - 1) : (phase == 1 ? 4 * (b.ib + 1) : 8);
}

template <typename T>
__device__ void body_corner_item(const DevBlock<T>& b, const PhysParams& P, int phase, int t) {
  const long long N = b.N;
  const int il = b.il, jl = b.jl, kl = b.kl, ie = b.ie, je = b.je, ke = b.ke;
  const T gamma = (T)P.gamma;
  auto C3 = [&](int i, int j, int k) { return cidx(b.Pi, b.Pj, i, j, k); };
  auto set3 = [&](long long d, long long a, long long bb, long long cc) {
    T wv[5];
    for (int v = 0; v < 5; v++) {
      wv[v] = b.w[v * N + a] + b.w[v * N + bb] - b.w[v * N + cc];
      b.w[v * N + d] = wv[v];
    }
    b.p[d] = depvars(gamma, wv);
  };
  if (phase == 0) {  // edges along k (k = 2..kl) and along j (j = 2..jl)
    if (t < 4 * (kl - 1)) {
      int k = 2 + t / 4, e = t % 4;
      if (e == 0) set3(C3(1, 1, k), C3(2, 1, k), C3(1, 2, k), C3(2, 2, k));
      else if (e == 1) set3(C3(ie, 1, k), C3(il, 1, k), C3(ie, 2, k), C3(il, 2, k));
      else if (e == 2) set3(C3(1, je, k), C3(2, je, k), C3(1, jl, k), C3(2, jl, k));
      else set3(C3(ie, je, k), C3(il, je, k), C3(ie, jl, k), C3(il, jl, k));
    } else {
      int u = t - 4 * (kl - 1);
      int j = 2 + u / 4, e = u % 4;
      if (e == 0) set3(C3(1, j, 1), C3(2, j, 1), C3(1, j, 2), C3(2, j, 2));
      else if (e == 1) set3(C3(ie, j, 1), C3(il, j, 1), C3(ie, j, 2), C3(il, j, 2));
      else if (e == 2) set3(C3(1, j, ke), C3(2, j, ke), C3(1, j, kl), C3(2, j, kl));
      else set3(C3(ie, j, ke), C3(il, j, ke), C3(ie, j, kl), C3(il, j, kl));
    }
  } else if (phase == 1) {  // edges along i (i = 0..ib)
    int i = t / 4, e = t % 4;
    if (e == 0) set3(C3(i, 1, 1), C3(i, 1, 2), C3(i, 2, 1), C3(i, 2, 2));
    else if (e == 1) set3(C3(i, 1, ke), C3(i, 2, ke), C3(i, 1, kl), C3(i, 2, kl));
    else if (e == 2) set3(C3(i, je, 1), C3(i, je, 1), C3(i, jl, 2), C3(i, jl, 2));  // bc_corner.f90:120 as written
    else set3(C3(i, je, ke), C3(i, jl, ke), C3(i, je, kl), C3(i, jl, kl));
  } else {  // the 8 corners; each reads only edge cells
    long long d, a, bq, cq, dq;
    switch (t) {
      case 0: d = C3(1, 1, 1); a = C3(2, 1, 1); bq = C3(1, 2, 1); cq = C3(1, 1, 2); dq = C3(2, 2, 2); break;
      case 1: d = C3(1, 1, ke); a = C3(2, 1, ke); bq = C3(1, 2, ke); cq = C3(1, 1, kl); dq = C3(2, 2, kl); break;
      case 2: d = C3(1, je, 1); a = C3(2, je, 1); bq = C3(1, jl, 1); cq = C3(1, je, 2); dq = C3(2, jl, 2); break;
      case 3: d = C3(ie, 1, 1); a = C3(il, 1, 1); bq = C3(ie, 2, 1); cq = C3(ie, 1, 2); dq = C3(il, 2, 2); break;
      case 4: d = C3(ie, 1, ke); a = C3(il, 1, ke); bq = C3(ie, 2, ke); cq = C3(ie, 1, kl); dq = C3(il, 2, kl); break;
      case 5: d = C3(ie, je, 1); a = C3(il, je, 1); bq = C3(ie, jl, 1); cq = C3(ie, je, 2); dq = C3(il, jl, 2); break;
      case 6: d = C3(1, je, ke); a = C3(2, je, ke); bq = C3(1, jl, ke); cq = C3(1, je, kl); dq = C3(2, jl, kl); break;
      default: d = C3(ie, je, ke); a = C3(il, je, ke); bq = C3(ie, jl, ke); cq = C3(ie, je, kl); dq = C3(il, jl, kl); break;
    }
    T wv[5];
    for (int v = 0; v < 5; v++) {
      wv[v] = (b.w[v * N + a] + b.w[v * N + bq] + b.w[v * N + cq]) * T(2) / T(3) - b.w[v * N + dq];
      b.w[v * N + d] = wv[v];
    }
    b.p[d] = depvars(gamma, wv);
  }
}


template <typename T>
__global__ void k_bc_corner(DevBlock<T> b, PhysParams P, int phase) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < corner_items(b, phase)) body_corner_item(b, P, phase, t);
}

// the whole of bcond.f90 in one cooperative launch: the three face passes and
// the three corner phases with a grid barrier between them
template <typename T>
__global__ void __launch_bounds__(256, 2) k_bcond_coop(DevBlock<T> b, PhysParams P) {
  cg::grid_group g = cg::this_grid();
  const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long gs = (long long)gridDim.x * blockDim.x;
  const long long nf = bc_pass_items(b);
  for (int pass = 0; pass < 3; pass++) {
    for (long long t = gt; t < nf; t += gs) body_bc_pass(b, P, pass, t);
    g.sync();
  }
  for (int phase = 0; phase < 3; phase++) {
    const int n = corner_items(b, phase);
    for (long long t = gt; t < n; t += gs) body_corner_item(b, P, phase, (int)t);
    if (phase < 2) g.sync();
  }
}

// --------------------------------------------------------------- residual norm (euler.f90:431-447)
// Deterministic: fixed partial ranges, fixed-order tree per block, one final block.
constexpr int RT_THREADS = 256;
int rtrms_partials(long long ncells) {
  long long per = (long long)RT_THREADS * 8;
  long long n = (ncells + per - 1) / per;
  return (int)(n < 1 ? 1 : (n > 4096 ? 4096 : n));
}

template <typename T>
__device__ void body_rtrms_partial(const DevBlock<T>& b, double cfl, int vt, double* partial, int npart, int part) {
  __shared__ double sh[RT_THREADS];
  const long long tot = (long long)b.nx * b.ny * b.nz;
  const long long per = (tot + npart - 1) / npart;
  const long long lo = (long long)part * per, hi = min(tot, lo + per);
  double acc = 0.0;
  for (long long t = lo + threadIdx.x; t < hi; t += blockDim.x) {
    // 32-bit index arithmetic while the block's cells fit (the same cells)
    int i, j, k;
    if (tot < (1ll << 31)) {
      const int t32 = (int)t, nxy = b.nx * b.ny;
      k = t32 / nxy;
      const int r = t32 - k * nxy;
      j = r / b.nx;
      i = r - j * b.nx;
      i += 2, j += 2, k += 2;
    } else {
      i = 2 + (int)(t % b.nx);
      j = 2 + (int)((t / b.nx) % b.ny);
      k = 2 + (int)(t / ((long long)b.nx * b.ny));
    }
    long long c = cidx(b.Pi, b.Pj, i, j, k);
    double de = smul(cfl, (double)(vt ? *b.dtim : b.vdtim[c]));
    double rt = 0.0;
    if (b.blank[c] != 0) rt = sdiv((double)b.dw[c], de);
    acc = acc + smul(rt, rt);
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = RT_THREADS / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = sh[threadIdx.x] + sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[part] = sh[0];
  __syncthreads();
}

template <typename T>
__global__ void k_rtrms_partial(DevBlock<T> b, double cfl, int vt, double* partial, int npart) {
  body_rtrms_partial(b, cfl, vt, partial, npart, blockIdx.x);
}

// The partial sums in a fixed order by one warp: lane l adds the partials
// l, l+32, l+64, ... in turn, then the lanes' sums fold in a fixed halving
// tree.  A NaN norm is the stop of solver.f90:180, recorded in launch order
// like the kernels' other stops (err may be null).  Every lane of warp 0
// calls it.
__device__ __forceinline__ void body_rtrms_final(const double* partial, int npart, double ncell, double* out,
                                                 unsigned* err) {
  const int lane = threadIdx.x & 31;
  double a = 0.0;
  for (int q = lane; q < npart; q += 32) a = a + partial[q];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a = a + __shfl_down_sync(0xffffffffu, a, o);
  if (lane == 0) {
    const double r = sqrt(a / ncell);
    *out = r;
    if (err && r != r) atomicCAS(err, 0u, (unsigned)ERR_NANRES);
  }
}

__global__ void k_rtrms_final(const double* partial, int npart, double ncell, double* out, unsigned* err) {
  if (blockIdx.x == 0 && threadIdx.x < 32) body_rtrms_final(partial, npart, ncell, out, err);
}

// --------------------------------------------------------------- small whole-array kernels
template <typename T>
__device__ __forceinline__ void body_depvars(const DevBlock<T>& b, double gamma, long long c) {
  if (c >= b.N) return;
  T wv[5];
  for (int v = 0; v < 5; v++) wv[v] = b.w[v * b.N + c];
  b.p[c] = depvars((T)gamma, wv);
}
template <typename T>
__global__ void k_depvars_all(DevBlock<T> b, double gamma) {
  body_depvars(b, gamma, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

template <typename T>
__global__ void k_copy5(const T* __restrict__ src, T* __restrict__ dst, long long n) {
  long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) dst[c] = src[c];
}

// wn = w on physical cells, dw = fw = 0 everywhere (euler.f90:80-89)
template <typename T>
__device__ __forceinline__ void body_save_wn(const DevBlock<T>& b, long long c) {
  const long long N = b.N;
  int i = (int)(c % b.Pi);
  int j = (int)((c / b.Pi) % b.Pj);
  int k = (int)(c / ((long long)b.Pi * b.Pj));
  bool phys = i >= 2 && i <= b.il && j >= 2 && j <= b.jl && k >= 2 && k <= b.kl;
  for (int v = 0; v < 5; v++) {
    if (phys) b.wn[v * N + c] = b.w[v * N + c];
    b.dw[v * N + c] = T(0);
    b.fw[v * N + c] = T(0);
  }
}

template <typename T>
__global__ void k_save_wn(DevBlock<T> b) {
  long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < b.N) body_save_wn(b, c);
}

// wn = w on physical cells only (movco.f90:29-35)
template <typename T>
__device__ __forceinline__ void body_copy_wn(const DevBlock<T>& b, long long c) {
  if (c >= b.N) return;
  int i = (int)(c % b.Pi);
  int j = (int)((c / b.Pi) % b.Pj);
  int k = (int)(c / ((long long)b.Pi * b.Pj));
  if (!(i >= 2 && i <= b.il && j >= 2 && j <= b.jl && k >= 2 && k <= b.kl)) return;
  for (int v = 0; v < 5; v++) b.wn[v * b.N + c] = b.w[v * b.N + c];
}
template <typename T>
__global__ void k_copy_wn(DevBlock<T> b) {
  body_copy_wn(b, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

template <typename T>
__global__ void k_init_free(DevBlock<T> b, PhysParams P) {
  long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= b.N) return;
  const long long N = b.N;
  double rho0 = P.rho0;
  b.w[c] = (T)rho0;
  b.w[N + c] = (T)(rho0 * P.u0[0]);
  b.w[2 * N + c] = (T)(rho0 * P.u0[1]);
  b.w[3 * N + c] = (T)(rho0 * P.u0[2]);
  b.w[4 * N + c] = (T)P.e0;  // rho0*h0 - p0, init_flow.f90:59
}

// --------------------------------------------------------------- multigrid transfers
__device__ __forceinline__ void trilinear_factor(double x, double y, double z, double* fac) {
  fac[0] = (1.0 - x) * (1.0 - y) * (1.0 - z);
  fac[1] = x * (1.0 - y) * (1.0 - z);
  fac[2] = (1.0 - x) * y * (1.0 - z);
  fac[3] = x * y * (1.0 - z);
  fac[4] = (1.0 - x) * (1.0 - y) * z;
  fac[5] = x * (1.0 - y) * z;
  fac[6] = (1.0 - x) * y * z;
  fac[7] = x * y * z;
}

struct Xfer {
  int r[3], o[3];
  double rinv[3];  // 1/r when r is a power of two (x/r = x*(1/r) exactly), else 0
};

// collc.f90:58-158 for the coarse cells under one child
template <typename TC, typename TF>
__device__ __forceinline__ long long collc_items(const DevBlock<TC>&, const DevBlock<TF>& f, const Xfer& X) {
  return (long long)(f.nx / X.r[0]) * (f.ny / X.r[1]) * (f.nz / X.r[2]);
}
template <typename TC, typename TF>
__device__ __forceinline__ void body_collc(const DevBlock<TC>& c, const DevBlock<TF>& f, const Xfer& X,
                                           uint8_t* marker, long long t) {
  const int n0 = f.nx / X.r[0], n1 = f.ny / X.r[1], n2 = f.nz / X.r[2];
  if (t >= (long long)n0 * n1 * n2) return;
  int ic[3] = {X.o[0] + 2 + (int)(t % n0), X.o[1] + 2 + (int)((t / n0) % n1), X.o[2] + 2 + (int)(t / ((long long)n0 * n1))};
  if (ic[0] < 2 || ic[0] > c.il || ic[1] < 2 || ic[1] > c.jl || ic[2] < 2 || ic[2] > c.kl) return;
  const int lf[3] = {f.il, f.jl, f.kl};
  if constexpr (std::is_same<TC, float>::value && std::is_same<TF, double>::value) {
    // the mixed form's restriction from the FP64 finest level onto an FP32
    // level: the values land in FP32 storage, so the averages are formed in
    // FP32 (the same stencil; the 2:1 weights are exact in FP32)
    int sf[3];
    float xf[3];
    for (int d = 0; d < 3; d++) {
      const float tt = ((float)ic[d] - 1.5f - (float)X.o[d]) * (float)X.r[d];
      int s = (int)floorf(tt + 1.5f);
      s = s < 2 ? 2 : (s > lf[d] - 1 ? lf[d] - 1 : s);
      sf[d] = s;
      xf[d] = tt + 1.5f - (float)s;
    }
    const float wx[2] = {1.0f - xf[0], xf[0]}, wy[2] = {1.0f - xf[1], xf[1]}, wz[2] = {1.0f - xf[2], xf[2]};
    const long long cc = cidx(c.Pi, c.Pj, ic[0], ic[1], ic[2]);
    for (int v = 0; v < 5; v++) {
      float ar = 0.0f, aw = 0.0f;
      for (int dk = 0; dk < 2; dk++)
        for (int dj = 0; dj < 2; dj++)
          for (int di = 0; di < 2; di++) {
            const long long fq = cidx(f.Pi, f.Pj, sf[0] + di, sf[1] + dj, sf[2] + dk);
            const float wt = wx[di] * wy[dj] * wz[dk];
            ar = fmaf((float)f.dw[v * f.N + fq] * f.rvolf, wt, ar);
            aw = fmaf((float)f.w[v * f.N + fq], wt, aw);
          }
      c.wr[v * c.N + cc] = ar * (float)c.vol;
      c.w[v * c.N + cc] = aw;
    }
    marker[cc] = 1;
    return;
  }
  int sh[3];
  double xi[3];
  for (int d = 0; d < 3; d++) {
    double tt = ((double)ic[d] - 1.5 - (double)X.o[d]) * (double)X.r[d];
    int s = (int)floor(tt + 1.5);
    if (s < 2) s = 2;
    if (s > lf[d] - 1) s = lf[d] - 1;
    sh[d] = s;
    xi[d] = tt + 1.5 - (double)s;
  }
  double fac[8];
  trilinear_factor(xi[0], xi[1], xi[2], fac);
  const long long cc = cidx(c.Pi, c.Pj, ic[0], ic[1], ic[2]);
  for (int v = 0; v < 5; v++) {
    double acc = 0.0;
    int nn = 0;
    for (int dk = 0; dk < 2; dk++)
      for (int dj = 0; dj < 2; dj++)
        for (int di = 0; di < 2; di++) {
          long long fq = cidx(f.Pi, f.Pj, sh[0] + di, sh[1] + dj, sh[2] + dk);
          double val = smdiv((double)f.dw[v * f.N + fq], f.vol, f.rvol);
          acc = acc + (dk ? smul(val, fac[nn]) : val * fac[nn]);
          nn++;
        }
    c.wr[v * c.N + cc] = (TC)(acc * c.vol);
    acc = 0.0;
    nn = 0;
    for (int dk = 0; dk < 2; dk++)
      for (int dj = 0; dj < 2; dj++)
        for (int di = 0; di < 2; di++) {
          long long fq = cidx(f.Pi, f.Pj, sh[0] + di, sh[1] + dj, sh[2] + dk);
          acc = acc + (dk ? smul((double)f.w[v * f.N + fq], fac[nn]) : (double)f.w[v * f.N + fq] * fac[nn]);
          nn++;
        }
    c.w[v * c.N + cc] = (TC)acc;
  }
  marker[cc] = 1;
}
template <typename TC, typename TF>
__global__ void k_collc(DevBlock<TC> c, DevBlock<TF> f, Xfer X, uint8_t* marker) {
  body_collc(c, f, X, marker, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

__device__ __forceinline__ bool fine_to_coarse(const Xfer& X, int ncp0, int ncp1, int ncp2, int lc0, int lc1, int lc2,
                                               int i, int j, int k, int* sh, double* fac) {
  int ic[3] = {i, j, k};
  int nc[3] = {ncp0, ncp1, ncp2};
  int lc[3] = {lc0, lc1, lc2};
  double xi[3];
  for (int d = 0; d < 3; d++) {
    const double x = (double)ic[d] - 1.5;
    double u = (double)X.o[d] + (X.rinv[d] > 0.0 ? x * X.rinv[d] : x / (double)X.r[d]);
    if (u < 0.0 || u >= (double)nc[d]) return false;
    int s = (int)floor(u + 1.5);
    if (s < 2) s = 2;
    if (s > lc[d] - 1) s = lc[d] - 1;
    sh[d] = s;
    xi[d] = u + 1.5 - (double)s;
  }
  trilinear_factor(xi[0], xi[1], xi[2], fac);
  return true;
}

// the coarse correction w_c - ws_c of every coarse cell, formed once for the
// 64 fine cells whose interpolation takes it (the same subtraction)
template <typename TC>
__device__ __forceinline__ void body_addw_diff(const DevBlock<TC>& c, double* dc, long long q) {
  if (q >= c.N) return;
#pragma unroll
  for (int v = 0; v < 5; v++) dc[v * c.N + q] = (double)c.w[v * c.N + q] - (double)c.ws[v * c.N + q];
}
template <typename TC>
__global__ void k_addw_diff(DevBlock<TC> c, double* dc) {
  body_addw_diff(c, dc, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// addw.f90:83-188: w_f = store_w + I(w_c - ws_c), or I(w_c) in the FMG step;
// dc holds w_c - ws_c (k_addw_diff) unless fmg
template <typename TF, typename TC>
__device__ __forceinline__ void body_addw(const DevBlock<TF>& f, const DevBlock<TC>& c, const Xfer& X, int fmg,
                                          const double* dc, long long t) {
  if (t >= (long long)f.nx * f.ny * f.nz) return;
  int i = 2 + (int)(t % f.nx), j = 2 + (int)((t / f.nx) % f.ny), k = 2 + (int)(t / ((long long)f.nx * f.ny));
  if constexpr (std::is_same<TF, double>::value && std::is_same<TC, float>::value) {
    // the mixed form's finest level under an FP32 coarse level: the coarse
    // correction is FP32, so it is interpolated in FP32 (the same stencil
    // and weights, exact in FP32 for power-of-two ratios) and added to the
    // FP64 state in FP64
    if (!fmg) {
      const int ic[3] = {i, j, k}, nc[3] = {c.nx, c.ny, c.nz}, lc[3] = {c.il, c.jl, c.kl};
      int sf[3];
      float xf[3];
      for (int d = 0; d < 3; d++) {
        const float x = (float)ic[d] - 1.5f;
        const float u = (float)X.o[d] + (X.rinv[d] > 0.0 ? x * (float)X.rinv[d] : x / (float)X.r[d]);
        if (u < 0.0f || u >= (float)nc[d]) return;
        int s = (int)floorf(u + 1.5f);
        s = s < 2 ? 2 : (s > lc[d] - 1 ? lc[d] - 1 : s);
        sf[d] = s;
        xf[d] = u + 1.5f - (float)s;
      }
      const long long q = cidx(f.Pi, f.Pj, i, j, k);
      if (f.blank[q] == 0) return;
      const float wx[2] = {1.0f - xf[0], xf[0]}, wy[2] = {1.0f - xf[1], xf[1]}, wz[2] = {1.0f - xf[2], xf[2]};
      for (int v = 0; v < 5; v++) {
        float acc = 0.0f;
        for (int dk = 0; dk < 2; dk++)
          for (int dj = 0; dj < 2; dj++)
            for (int di = 0; di < 2; di++) {
              const long long cq = cidx(c.Pi, c.Pj, sf[0] + di, sf[1] + dj, sf[2] + dk);
              acc = fmaf((float)dc[v * c.N + cq], wx[di] * wy[dj] * wz[dk], acc);
            }
        f.w[v * f.N + q] = f.w[v * f.N + q] + (double)acc;
      }
      return;
    }
  }
  int sh[3];
  double fac[8];
  if (!fine_to_coarse(X, c.nx, c.ny, c.nz, c.il, c.jl, c.kl, i, j, k, sh, fac)) return;
  const long long q = cidx(f.Pi, f.Pj, i, j, k);
  if (f.blank[q] == 0) return;
  for (int v = 0; v < 5; v++) {
    double acc = 0.0;
    int nn = 0;
    for (int dk = 0; dk < 2; dk++)
      for (int dj = 0; dj < 2; dj++)
        for (int di = 0; di < 2; di++) {
          long long cq = cidx(c.Pi, c.Pj, sh[0] + di, sh[1] + dj, sh[2] + dk);
          double val = fmg ? (double)c.w[v * c.N + cq] : dc[v * c.N + cq];
          // half the products on the integer pipes (smul), half on the FP64 pipe
          acc = acc + (dk ? smul(val, fac[nn]) : val * fac[nn]);
          nn++;
        }
    if (fmg)
      f.w[v * f.N + q] = (TF)acc;
    else
      f.w[v * f.N + q] = (TF)((double)f.w[v * f.N + q] + acc);
  }
}
template <typename TF, typename TC>
__global__ void k_addw(DevBlock<TF> f, DevBlock<TC> c, Xfer X, int fmg, const double* dc) {
  body_addw(f, c, X, fmg, dc, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// bc_overlap.f90:32-90: ghost cell dst[t] of block g takes the trilinear
// interpolation of partner p's state from the 2x2x2 cells at src[t] (its
// physical cells: no cell is both read and written), then depvars
template <typename T>
__global__ void k_overlap(DevBlock<T> g, DevBlock<T> p, const long long* __restrict__ dst,
                          const long long* __restrict__ src, const double* __restrict__ fac, long long n,
                          double gamma) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const long long q = dst[t], s = src[t];
  const long long sj = p.Pi, sk = (long long)p.Pi * p.Pj;
  const double* f = fac + 8 * t;
  T wv[5];
#pragma unroll
  for (int v = 0; v < 5; v++) {
    double acc = 0.0;
    int nn = 0;
    for (int dk = 0; dk < 2; dk++)
      for (int dj = 0; dj < 2; dj++)
        for (int di = 0; di < 2; di++) acc = acc + (double)p.w[v * p.N + s + di + dj * sj + dk * sk] * f[nn++];
    wv[v] = (T)acc;
    g.w[v * g.N + q] = wv[v];
  }
  g.p[q] = depvars((T)gamma, wv);
}

// bc_embed.f90:47-143: fine ghost cells whose centre lies in the parent
template <typename TF, typename TC>
__device__ __forceinline__ void body_embed(const DevBlock<TF>& f, const DevBlock<TC>& c, const Xfer& X, double gamma,
                                           long long t) {
  if (t >= f.N) return;
  int i = (int)(t % f.Pi), j = (int)((t / f.Pi) % f.Pj), k = (int)(t / ((long long)f.Pi * f.Pj));
  if (i >= 2 && i <= f.il && j >= 2 && j <= f.jl && k >= 2 && k <= f.kl) return;
  int sh[3];
  double fac[8];
  if (!fine_to_coarse(X, c.nx, c.ny, c.nz, c.il, c.jl, c.kl, i, j, k, sh, fac)) return;
  const long long q = t;
  TF wv[5];
  for (int v = 0; v < 5; v++) wv[v] = f.w[v * f.N + q];
  if (f.blank[q] != 0) {
    for (int v = 0; v < 5; v++) {
      double acc = 0.0;
      int nn = 0;
      for (int dk = 0; dk < 2; dk++)
        for (int dj = 0; dj < 2; dj++)
          for (int di = 0; di < 2; di++)
            acc = acc + (double)c.w[v * c.N + cidx(c.Pi, c.Pj, sh[0] + di, sh[1] + dj, sh[2] + dk)] * fac[nn++];
      wv[v] = (TF)acc;
      f.w[v * f.N + q] = wv[v];
    }
  }
  f.p[q] = depvars((TF)gamma, wv);
}
template <typename TF, typename TC>
__global__ void k_embed(DevBlock<TF> f, DevBlock<TC> c, Xfer X, double gamma) {
  body_embed(f, c, X, gamma, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// upload_solut.f90:203-237: the cell-centre output variables of the physical
// cells, solut(2:il,2:jl,2:kl,1:nval) in Fortran order (nval 7, or 11 with
// the NS energy and three zero gradients); the expressions in the
// reference's order, in FP64 whatever the block's storage
template <typename T>
__global__ void k_solut(DevBlock<T> b, double gamma, double p0, double rm, double p_tot, int ns, double* out) {
  const long long ncell = (long long)b.nx * b.ny * b.nz;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncell) return;
  const int i = 2 + (int)(t % b.nx), j = 2 + (int)((t / b.nx) % b.ny), k = 2 + (int)(t / ((long long)b.nx * b.ny));
  const long long N = b.N, c = cidx(b.Pi, b.Pj, i, j, k);
  const double rr = (double)b.w[c];
  const double uu = (double)b.w[N + c] / rr;
  const double vv = (double)b.w[2 * N + c] / rr;
  const double ww = (double)b.w[3 * N + c] / rr;
  const double re = (double)b.w[4 * N + c];
  const double qq = 0.5 * (uu * uu + vv * vv + ww * ww) * rr;
  double pp = (gamma - 1.0) * (re > qq ? re - qq : 0.0);  // dim(re, qq)
  const double mm = sqrt((uu * uu + vv * vv + ww * ww) / gamma / pp * rr);
  const double ptloss = pp * pow(1.0 + 0.2 * mm * mm, 3.5) / p_tot - 1.0;
  pp = (pp / p0 - 1.0) * 2.0 / (gamma * rm * rm);
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

// wall forces from the records (new): 7 sums, fixed order within one block.
// Pressure on each wall face and, when mu > 0 (NS), the wall's viscous
// stress: the momentum the solver's wall flux (rec_wall_terms) gives the
// fluid, with the opposite sign
template <typename T>
__global__ void k_forces(DevBlock<T> b, double ox, double oy, double oz, double hx, double hy, double hz, double cx,
                         double cy, double cz, double mu, double* out) {
  __shared__ double sh[7][256];
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  const double org[3] = {ox, oy, oz}, h[3] = {hx, hy, hz}, ctr[3] = {cx, cy, cz};
  for (int m = threadIdx.x; m < b.nmir; m += blockDim.x) {
    const int* ri = b.rec_i + 8 * m;
    if (ri[6] == 0) continue;  // a wall face another block of the level counts
    int ax = ri[4] - 1;
    double sgn = ri[3] >= 4 ? 1.0 : -1.0;
    long long c = cidx(b.Pi, b.Pj, ri[0], ri[1], ri[2]);
    double area = b.rec_area[m];
    double pw = 0.5 * ((double)b.p[c] + (double)b.rec_psol[m]);
    double fv[3] = {0, 0, 0};
    if (mu > 0.0) {  // visc_wall of rec_wall_terms, in FP64
      const bool plus = ri[3] >= 4;
      const double S = fabs(b.s[ax]), r0 = (double)b.w[c];
      for (int a = 0; a < 3; a++) {
        const double u = (double)b.w[(1 + a) * b.N + c] / r0;
        const double ug = 2.0 * b.rec_qb[3 * m + a] - u;
        const double gn = plus ? (ug - u) / h[ax] : (u - ug) / h[ax];
        const double tau = (a == ax) ? (4.0 / 3.0) * mu * gn : mu * gn;
        fv[a] = plus ? -(S * tau) : S * tau;
      }
    }
    double f[3];
    for (int d = 0; d < 3; d++) f[d] = (d == ax ? pw * area * sgn : 0.0) + fv[d];
    double xf[3];
    for (int d = 0; d < 3; d++) xf[d] = org[d] + ((double)ri[d] - 1.5) * h[d];
    xf[ax] = xf[ax] + sgn * 0.5 * h[ax];
    double r[3] = {xf[0] - ctr[0], xf[1] - ctr[1], xf[2] - ctr[2]};
    acc[0] += f[0];
    acc[1] += f[1];
    acc[2] += f[2];
    acc[3] += r[1] * f[2] - r[2] * f[1];
    acc[4] += r[2] * f[0] - r[0] * f[2];
    acc[5] += r[0] * f[1] - r[1] * f[0];
  }
  for (int q = 0; q < 6; q++) sh[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int q = 0; q < 6; q++) sh[q][threadIdx.x] += sh[q][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x < 6) out[threadIdx.x] = sh[threadIdx.x][0];
}

// =============================================================== one-launch-per-phase kernels
template <typename T, bool SLOPES, bool FAST = false>
__global__ void __launch_bounds__(256, SLOPES ? 3 : 6) k_prep(DevBlock<T> b, PhysParams P, int dissip_on) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < (long long)b.ie * b.je * b.ke) body_prep<T, SLOPES, FAST>(b, P, dissip_on, t);
}
// the velocities of every cell, ghosts included, into F[0..2] for the MUSCL
// Roe form (one reciprocal of the density and mdiv: the IEEE quotients)
template <typename T>
__global__ void k_prim(DevBlock<T> b) {
  long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= b.N) return;
  const long long N = b.N;
  const T r = b.w[c], y = T(1) / r;
#pragma unroll
  for (int a = 0; a < 3; a++) b.F[(long long)a * N + c] = mdiv(b.w[(long long)(1 + a) * N + c], r, y);
}
template <typename T>
__global__ void __launch_bounds__(256, 4) k_face(DevBlock<T> b, PhysParams P, int dissip_on, T cd) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < (long long)(b.ie - 1) * (b.je - 1) * (b.ke - 1)) body_face<T, FACE_CENTRAL>(b, P, dissip_on, cd, t);
}
template <typename T>
__global__ void __launch_bounds__(256, 6) k_face_jst(DevBlock<T> b, PhysParams P, int dissip_on, T cd) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < (long long)(b.ie - 1) * (b.je - 1) * (b.ke - 1)) body_face<T, FACE_JST>(b, P, dissip_on, cd, t);
}
// the contracted form's dissipation faces (no convective face fluxes)
template <typename T>
__global__ void __launch_bounds__(256, 4) k_face_diss(DevBlock<T> b, PhysParams P, T cd) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < (long long)(b.ie - 1) * (b.je - 1) * (b.ke - 1)) body_face_diss<T>(b, P, cd, t);
}
// the Roe faces (MUSCL states, upwind flux, and the viscous flux with NS)
template <typename T>
__global__ void __launch_bounds__(256, 3) k_face_roe(DevBlock<T> b, PhysParams P, int dissip_on, T cd) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < (long long)(b.ie - 1) * (b.je - 1) * (b.ke - 1)) body_face<T, FACE_ROE>(b, P, dissip_on, cd, t);
}
// a stage without dissipation of the central scheme: only the convective
// face fluxes efs(q) = 0.5*(F(q) + F(q-1)), the same expression as face_dir,
// in a kernel small enough to keep the memory system busy
template <typename T>
__device__ __forceinline__ void body_face_conv(const DevBlock<T>& b, long long t) {
  const int ex = b.ie - 1, ey = b.je - 1;
  if (t >= (long long)ex * ey * (b.ke - 1)) return;
  const int i = 2 + (int)(t % ex), j = 2 + (int)((t / ex) % ey), k = 2 + (int)(t / ((long long)ex * ey));
  const long long N = b.N, c = cidx(b.Pi, b.Pj, i, j, k);
  const bool on[3] = {j <= b.jl && k <= b.kl, i <= b.il && k <= b.kl, i <= b.il && j <= b.jl};
  const long long sts[3] = {1, (long long)b.Pi, (long long)b.Pi * b.Pj};
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (!on[d]) continue;
    const T* F = b.F + (long long)(d * 5) * N;
    T* E = b.efs + (long long)(d * 5) * N;
#pragma unroll
    for (int v = 0; v < 5; v++) E[v * N + c] = mulhalf(F[v * N + c] + F[v * N + c - sts[d]]);
  }
}
template <typename T>
__global__ void __launch_bounds__(256) k_face_conv(DevBlock<T> b) {
  body_face_conv(b, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}
template <typename T, bool FAST = false>
__global__ void k_combine(DevBlock<T> b, PhysParams P, StageArgs A, unsigned* err) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < (long long)b.nx * b.ny * b.nz) body_combine<T, FAST>(b, P, A, err, t);
}
template <typename T, typename TC, int D, bool SC = false>
__global__ void k_irs(DevBlock<T> b, IrsTables tb, TC bb) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < 5 * irs_lines<T, D>(b)) body_irs<T, TC, D, SC>(b, tb, bb, t);
}
template <typename T>
__global__ void k_update(DevBlock<T> b, PhysParams P, StageArgs A) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < (long long)b.nx * b.ny * b.nz) body_update(b, P, A, t);
}
template <typename T>
__global__ void k_cutcell(DevBlock<T> b, PhysParams P, unsigned* err) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  body_cutcell(b, P, err, m);
}
// =============================================================== one euler update in one launch
// For the small coarse grids of the multigrid hierarchy every phase of
// euler.f90 is latency-bound, so one cooperative kernel runs them all with a
// grid-wide barrier between phases instead of ~70 launches.
struct EulerArgs {
  int mstage;
  int do_timestep;   // timestep.f90 before euler (solver.f90:154,218)
  int lfir, lres, rt;
  int smoo_on;
  StageArgs st[8];
  IrsTables tab[3];
  double* rt_partial;
  int npart;
  double* rt_out;
  unsigned* err;
  unsigned long long* trace;  // optional: globaltimer after every barrier (block 0, thread 0)
};

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

template <typename T, typename TA>
__global__ void __launch_bounds__(256, 1) k_euler_coop(DevBlock<T> b, PhysParams P, EulerArgs E) {
  cg::grid_group g_ = cg::this_grid();
  int ntr = 0;
  struct Sync {
    cg::grid_group& g;
    unsigned long long* tr;
    int& n;
    __device__ void sync() {
      g.sync();
      if (tr && blockIdx.x == 0 && threadIdx.x == 0 && n < 255) tr[1 + n++] = gtimer();
    }
  } g{g_, E.trace, ntr};
  if (E.trace && blockIdx.x == 0 && threadIdx.x == 0) E.trace[0] = gtimer();
  // items go round-robin over the blocks (item q to block q mod G), so that
  // the few cells of a small level still spread over every SM's FP64 pipe
  const long long gt = (long long)threadIdx.x * gridDim.x + blockIdx.x;
  const long long gs = (long long)gridDim.x * blockDim.x;
  const long long ncell = (long long)b.nx * b.ny * b.nz;
  if (E.do_timestep) {
    if (gt == 0) *b.dtim = 10.0;
    g.sync();
    for (long long base = (long long)blockIdx.x * blockDim.x; base < ncell; base += gs) {
      long long t = base + threadIdx.x;
      unsigned long long mine = ~0ull;
      if (t < ncell) mine = body_timestep<T, TA>(b, P, E.err, t);
      block_min_to(mine, b.dtim);
    }
    g.sync();
  }
  if (E.lfir)
    for (long long q = gt; q < 5 * b.N; q += gs) b.ws[q] = b.w[q];
  for (long long q = gt; q < b.N; q += gs) body_save_wn(b, q);
  g.sync();
  const long long nprep = (long long)b.ie * b.je * b.ke;
  const long long nface = (long long)(b.ie - 1) * (b.je - 1) * (b.ke - 1);
  for (int m = 1; m <= E.mstage; m++) {
    const StageArgs& A = E.st[m - 1];
    if (A.fast) {
      for (long long t = gt; t < nprep; t += gs) body_prep<T, false, true>(b, P, A.dissip_on, t);
      g.sync();
      if (A.dissip_on)
        for (long long t = gt; t < nface; t += gs) body_face_diss(b, P, (T)A.cd, t);
    } else {
      for (long long t = gt; t < nprep; t += gs) body_prep(b, P, A.dissip_on, t);
      g.sync();
      for (long long t = gt; t < nface; t += gs) body_face(b, P, A.dissip_on, (T)A.cd, t);
    }
    for (long long t = gt; t < b.nmir; t += gs) rec_wall_terms(b, P, A.dissip_on, (T)A.cd, E.err, (int)t);
    g.sync();
    if (A.fast)
      for (long long t = gt; t < ncell; t += gs) body_combine<T, true>(b, P, A, E.err, t);
    else
      for (long long t = gt; t < ncell; t += gs) body_combine<T>(b, P, A, E.err, t);
    g.sync();
    if (E.lres) return;
    if (A.irs && P.irs_kind == 1) {
      for (long long t = gt; t < irs_lines<T, 0>(b); t += gs) body_psmoo_line<T, TA, 0>(b, t);
      g.sync();
      for (long long t = gt; t < irs_lines<T, 1>(b); t += gs) body_psmoo_line<T, TA, 1>(b, t);
      g.sync();
      for (long long t = gt; t < irs_lines<T, 2>(b); t += gs) body_psmoo_line<T, TA, 2>(b, t);
      g.sync();
    } else if (A.irs) {
      const TA bb = (TA)(-P.smoo);
      for (long long t = gt; t < 5 * irs_lines<T, 0>(b); t += gs) body_irs<T, TA, 0>(b, E.tab[0], bb, t);
      g.sync();
      for (long long t = gt; t < 5 * irs_lines<T, 1>(b); t += gs) body_irs<T, TA, 1>(b, E.tab[1], bb, t);
      g.sync();
      for (long long t = gt; t < 5 * irs_lines<T, 2>(b); t += gs) body_irs<T, TA, 2>(b, E.tab[2], bb, t);
      g.sync();
    }
    if (A.irs) {
      for (long long t = gt; t < ncell; t += gs) body_update(b, P, A, t);
      g.sync();
    }
    for (long long t = gt; t < b.nmir; t += gs) body_cutcell(b, P, E.err, (int)t);
    g.sync();
    for (int pass = 0; pass < 3; pass++) {
      const long long nf = bc_pass_items(b);
      for (long long t = gt; t < nf; t += gs) body_bc_pass(b, P, pass, t);
      g.sync();
    }
    for (int phase = 0; phase < 3; phase++) {
      const int n = corner_items(b, phase);
      for (long long t = gt; t < n; t += gs) body_corner_item(b, P, phase, (int)t);
      g.sync();
    }
  }
  if (E.rt) {
    for (int part = blockIdx.x; part < E.npart; part += gridDim.x)
      body_rtrms_partial(b, P.cfl, P.vt, E.rt_partial, E.npart, part);
    g.sync();
    if (blockIdx.x == 0 && threadIdx.x < 32) body_rtrms_final(E.rt_partial, E.npart, (double)ncell, E.rt_out, E.err);
  }
  if (E.trace && blockIdx.x == 0 && threadIdx.x == 0) E.trace[255] = (unsigned long long)ntr;
}

// =============================================================== several cases in one launch
// The same phase of a group of cases in one launch: the cases' work items
// laid end to end, each case's range rounded up to whole 256-thread blocks,
// so that a thread block serves one case (the per-block reductions of the
// time step minimum and the residual partial sums stay within a case).
// Each case runs the same bodies in the same order as alone, so its results
// are those of its own launches.
template <typename T>
struct MultiArgs {
  const DevBlock<T>* B;
  const PhysParams* P;
  unsigned* const* err;
  const IrsTables* tab;
  double* const* rt_partial;
  const int* npart;
  double* const* rt_out;
  const long long* off;
  int nc;
};

__device__ __forceinline__ int multi_case(const long long* off, int nc, long long base) {
  __shared__ int sq;
  if (threadIdx.x == 0) {
    int q = 0;
    while (q + 1 < nc && off[q + 1] <= base) q++;
    sq = q;
  }
  __syncthreads();
  return sq;
}

template <typename T, typename F>
__global__ void __launch_bounds__(256) k_multi(MultiArgs<T> M, F f) {
  const long long base = (long long)blockIdx.x * 256;
  const int q = multi_case(M.off, M.nc, base);
  f(M, q, base - M.off[q] + threadIdx.x);
}

template <typename T> struct FDtimReset {
  __device__ void operator()(const MultiArgs<T>& M, int q, long long t) const {
    if (t == 0) *M.B[q].dtim = 10.0;
  }
};
template <typename T, typename TC> struct FTimestep {
  __device__ void operator()(const MultiArgs<T>& M, int q, long long t) const {
    const DevBlock<T>& b = M.B[q];
    unsigned long long mine = ~0ull;
    if (t < (long long)b.nx * b.ny * b.nz) mine = body_timestep<T, TC>(b, M.P[q], M.err[q], t);
    block_min_to(mine, b.dtim);
  }
};
template <typename T> struct FCopyWs {
  __device__ void operator()(const MultiArgs<T>& M, int q, long long t) const {
    const DevBlock<T>& b = M.B[q];
    if (t < 5 * b.N) b.ws[t] = b.w[t];
  }
};
template <typename T> struct FSaveWn {
  __device__ void operator()(const MultiArgs<T>& M, int q, long long t) const {
    if (t < M.B[q].N) body_save_wn(M.B[q], t);
  }
};
template <typename T, bool FAST> struct FPrep {
  int dissip_on;
  __device__ void operator()(const MultiArgs<T>& M, int q, long long t) const {
    const DevBlock<T>& b = M.B[q];
    if (t < (long long)b.ie * b.je * b.ke) body_prep<T, false, FAST>(b, M.P[q], dissip_on, t);
  }
};
template <typename T> struct FFace {
  int dissip_on;
  T cd;
  __device__ void operator()(const MultiArgs<T>& M, int q, long long t) const {
    const DevBlock<T>& b = M.B[q];
    if (t < (long long)(b.ie - 1) * (b.je - 1) * (b.ke - 1)) body_face<T, FACE_CENTRAL>(b, M.P[q], dissip_on, cd, t);
  }
};
template <typename T> struct FFaceConv {
  __device__ void operator()(const MultiArgs<T>& M, int q, long long t) const { body_face_conv(M.B[q], t); }
};
template <typename T> struct FFaceDiss {
  T cd;
  __device__ void operator()(const MultiArgs<T>& M, int q, long long t) const {
    const DevBlock<T>& b = M.B[q];
    if (t < (long long)(b.ie - 1) * (b.je - 1) * (b.ke - 1)) body_face_diss<T>(b, M.P[q], cd, t);
  }
};
template <typename T> struct FRec {
  int dissip_on;
  T cd;
  __device__ void operator()(const MultiArgs<T>& M, int q, long long t) const {
    if (t < M.B[q].nmir) rec_wall_terms(M.B[q], M.P[q], dissip_on, cd, M.err[q], (int)t);
  }
};
template <typename T, bool FAST> struct FCombine {
  StageArgs A;
  __device__ void operator()(const MultiArgs<T>& M, int q, long long t) const {
    const DevBlock<T>& b = M.B[q];
    if (t < (long long)b.nx * b.ny * b.nz) body_combine<T, FAST>(b, M.P[q], A, M.err[q], t);
  }
};
template <typename T, typename TC, int D> struct FIrs {
  __device__ void operator()(const MultiArgs<T>& M, int q, long long t) const {
    const DevBlock<T>& b = M.B[q];
    if (t < 5 * irs_lines<T, D>(b)) body_irs<T, TC, D>(b, M.tab[3 * q + D], (TC)(-M.P[q].smoo), t);
  }
};
// the mixed form's finest level: FP32 sweeps on one FP32 copy of dw (in F)
template <typename TS, typename TO, int D> struct FIrsMixed {
  __device__ void operator()(const MultiArgs<double>& M, int q, long long t) const {
    const DevBlock<double>& b = M.B[q];
    if (t >= 5 * irs_lines<double, D>(b)) return;
    float* cp = (float*)b.F;
    const TS* src = D == 0 ? (const TS*)b.dw : (const TS*)cp;
    TO* out = D == 2 ? (TO*)b.dw : (TO*)cp;
    body_irs_mixed<TS, TO, D>(b, M.tab[3 * q + D], (float)(-M.P[q].smoo), src, cp, out, t);
  }
};
template <typename T> struct FUpdate {
  StageArgs A;
  __device__ void operator()(const MultiArgs<T>& M, int q, long long t) const {
    const DevBlock<T>& b = M.B[q];
    if (t < (long long)b.nx * b.ny * b.nz) body_update(b, M.P[q], A, t);
  }
};
template <typename T> struct FCutcell {
  __device__ void operator()(const MultiArgs<T>& M, int q, long long t) const {
    if (t < M.B[q].nmir) body_cutcell(M.B[q], M.P[q], M.err[q], (int)t);
  }
};
template <typename T> struct FBcPass {
  int pass;
  __device__ void operator()(const MultiArgs<T>& M, int q, long long t) const {
    if (t < bc_pass_items(M.B[q])) body_bc_pass(M.B[q], M.P[q], pass, t);
  }
};
template <typename T> struct FCorner {
  int phase;
  __device__ void operator()(const MultiArgs<T>& M, int q, long long t) const {
    if (t < corner_items(M.B[q], phase)) body_corner_item(M.B[q], M.P[q], phase, (int)t);
  }
};
template <typename T> struct FDepvars {
  __device__ void operator()(const MultiArgs<T>& M, int q, long long t) const { body_depvars(M.B[q], M.P[q].gamma, t); }
};
template <typename T> struct FCopyWn {
  __device__ void operator()(const MultiArgs<T>& M, int q, long long t) const { body_copy_wn(M.B[q], t); }
};
// residual partial sums: thread block (case, part), 256 threads each
template <typename T> struct FRtrmsPartial {
  __device__ void operator()(const MultiArgs<T>& M, int q, long long t) const {
    const int part = (int)(t / 256);
    if (part < M.npart[q]) body_rtrms_partial(M.B[q], M.P[q].cfl, M.P[q].vt, M.rt_partial[q], M.npart[q], part);
  }
};
template <typename T> struct FRtrmsFinal {
  __device__ void operator()(const MultiArgs<T>& M, int q, long long t) const {
    const DevBlock<T>& b = M.B[q];
    if (t < 32) body_rtrms_final(M.rt_partial[q], M.npart[q], (double)b.nx * b.ny * b.nz, M.rt_out[q], M.err[q]);
  }
};

// the transfers between the levels of a group: child f and parent c of each case
template <typename TC, typename TF>
struct MultiPairArgs {
  const DevBlock<TC>* C;
  const DevBlock<TF>* F;
  const Xfer* X;
  uint8_t* const* marker;
  double* const* dc;
  const PhysParams* P;
  const long long* off;
  int nc;
};
template <typename TC, typename TF, typename Fn>
__global__ void __launch_bounds__(256) k_multi2(MultiPairArgs<TC, TF> M, Fn f) {
  const long long base = (long long)blockIdx.x * 256;
  const int q = multi_case(M.off, M.nc, base);
  f(M, q, base - M.off[q] + threadIdx.x);
}
template <typename TC, typename TF> struct FMarkerClear {
  __device__ void operator()(const MultiPairArgs<TC, TF>& M, int q, long long t) const {
    if (t < M.C[q].N) M.marker[q][t] = 0;
  }
};
template <typename TC, typename TF> struct FCollc {
  __device__ void operator()(const MultiPairArgs<TC, TF>& M, int q, long long t) const {
    body_collc(M.C[q], M.F[q], M.X[q], M.marker[q], t);
  }
};
template <typename TC, typename TF> struct FAddwDiff {
  __device__ void operator()(const MultiPairArgs<TC, TF>& M, int q, long long t) const {
    body_addw_diff(M.C[q], M.dc[q], t);
  }
};
template <typename TC, typename TF> struct FAddw {
  int fmg;
  __device__ void operator()(const MultiPairArgs<TC, TF>& M, int q, long long t) const {
    body_addw(M.F[q], M.C[q], M.X[q], fmg, M.dc[q], t);
  }
};
template <typename TC, typename TF> struct FEmbed {
  __device__ void operator()(const MultiPairArgs<TC, TF>& M, int q, long long t) const {
    body_embed(M.F[q], M.C[q], M.X[q], M.P[q].gamma, t);
  }
};

// =============================================================== launchers
constexpr int TPB = 256;

// Threads per block for n work items: 256, halved down to 32 while the grid
// would not give every SM two blocks.  The stage kernels are bound by the FP64
// pipe of the SMs they run on, so on the small coarse levels spreading the
// cells over all SMs is worth more than wide blocks.
inline int tpb_for(long long n) {
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0) nsm = 152;
  }
  int t = TPB;
  while (t > 32 && n < (long long)t * nsm * 2) t >>= 1;
  return t;
}
#define LAUNCH_N(n) nblk((n), tpb_for(n)), tpb_for(n)

template <typename T>
void launch_solut(const DevBlock<T>& b, const PhysParams& P, double rm, double p_tot, int ns, double* out,
                  cudaStream_t s) {
  const long long n = (long long)b.nx * b.ny * b.nz;
  k_solut<T><<<nblk(n, TPB), TPB, 0, s>>>(b, P.gamma, P.p0, rm, p_tot, ns, out);
}


template <typename T>
void launch_timestep(const DevBlock<T>& b, const PhysParams& P, unsigned* err, cudaStream_t s, bool aux32) {
  long long n = (long long)b.nx * b.ny * b.nz;
  k_dtim_reset<<<1, 32, 0, s>>>(b.dtim);
  if (aux32)
    k_timestep<T, float><<<LAUNCH_N(n), 0, s>>>(b, P, err);
  else
    k_timestep<T, T><<<LAUNCH_N(n), 0, s>>>(b, P, err);
}

template <typename T>
void launch_stage_part(int part, const DevBlock<T>& b, const PhysParams& P, const StageArgs& A, unsigned* err,
                       cudaStream_t s) {
  if (part == 0) {
    long long n1 = (long long)b.ie * b.je * b.ke;
    if (A.fast) {
      k_prep<T, false, true><<<LAUNCH_N(n1), 0, s>>>(b, P, A.dissip_on);
    } else if (P.distype == 2) {
      k_prim<T><<<LAUNCH_N(b.N), 0, s>>>(b);
      k_prep<T, true><<<LAUNCH_N(n1), 0, s>>>(b, P, A.dissip_on);
    } else {
      k_prep<T, false><<<LAUNCH_N(n1), 0, s>>>(b, P, A.dissip_on);
    }
  } else if (part == 1) {
    long long n2 = (long long)(b.ie - 1) * (b.je - 1) * (b.ke - 1);
    if (A.fast) {
      if (A.dissip_on) k_face_diss<T><<<LAUNCH_N(n2), 0, s>>>(b, P, (T)A.cd);
    } else if (!A.dissip_on && P.distype == 0)
      k_face_conv<T><<<LAUNCH_N(n2), 0, s>>>(b);
    else if (P.distype == 0 && !P.eqn_ns && !P.matrix)
      k_face_jst<T><<<LAUNCH_N(n2), 0, s>>>(b, P, A.dissip_on, (T)A.cd);
    else if (P.distype == 0)
      k_face<T><<<LAUNCH_N(n2), 0, s>>>(b, P, A.dissip_on, (T)A.cd);
    else
      k_face_roe<T><<<LAUNCH_N(n2), 0, s>>>(b, P, A.dissip_on, (T)A.cd);
  } else if (part == 2) {
    if (b.nmir > 0) k_rec_wall<T><<<LAUNCH_N(b.nmir), 0, s>>>(b, P, A.dissip_on, (T)A.cd, err);
  } else if (part == 3) {
    long long n3 = (long long)b.nx * b.ny * b.nz;
    if (A.fast)
      k_combine<T, true><<<LAUNCH_N(n3), 0, s>>>(b, P, A, err);
    else
      k_combine<T><<<LAUNCH_N(n3), 0, s>>>(b, P, A, err);
  }
}

// One stage.  With a side stream and two events, the record pass runs on the
// side stream beside the face pass (it needs only the prep pass's output);
// the combine pass waits for both.
template <typename T>
void launch_stage(const DevBlock<T>& b, const PhysParams& P, const StageArgs& A, unsigned* err, cudaStream_t s,
                  cudaStream_t side, cudaEvent_t fork, cudaEvent_t join) {
  launch_stage_part<T>(0, b, P, A, err, s);
  const bool beside = b.nmir > 0 && side && fork && join;
  if (beside) {
    cudaEventRecord(fork, s);
    cudaStreamWaitEvent(side, fork, 0);
    launch_stage_part<T>(2, b, P, A, err, side);
    cudaEventRecord(join, side);
  } else {
    launch_stage_part<T>(2, b, P, A, err, s);
  }
  launch_stage_part<T>(1, b, P, A, err, s);
  if (beside) cudaStreamWaitEvent(s, join, 0);
  launch_stage_part<T>(3, b, P, A, err, s);
}

// the line-sweep variant: 0 = one thread per (line, variable) in global
// memory, 1 = shared-memory tiles of 64 lines; the autotuner picks per block
// and direction
template <typename T, typename TC, int D>
void launch_irs_dir(const DevBlock<T>& b, const IrsTables& tb, TC bb, cudaStream_t s, int variant) {
  const long long lines = D == 0 ? (long long)b.ny * b.nz : (D == 1 ? (long long)b.nx * b.nz : (long long)b.nx * b.ny);
  const int len = (D == 0 ? b.il : (D == 1 ? b.jl : b.kl)) - 1;
  constexpr int LT = 64;
  const size_t sm = irs_smem_bytes<TC, LT>(len | 1);
  if constexpr (D == 0 && std::is_same<T, float>::value && std::is_same<TC, float>::value) {
    const int kk = irs_scan_k(len);
    if (variant == 2 && kk) {  // one warp per (line, variable), in place
      const unsigned g = (unsigned)nblk(32 * 5 * lines, 256);
      float* out = (float*)b.dw;
      if (kk == 2) k_irs_scan_i<2, float><<<g, 256, 0, s>>>(b, tb, bb, out);
      if (kk == 4) k_irs_scan_i<4, float><<<g, 256, 0, s>>>(b, tb, bb, out);
      if (kk == 6) k_irs_scan_i<6, float><<<g, 256, 0, s>>>(b, tb, bb, out);
      if (kk == 8) k_irs_scan_i<8, float><<<g, 256, 0, s>>>(b, tb, bb, out);
      if (kk == 12) k_irs_scan_i<12, float><<<g, 256, 0, s>>>(b, tb, bb, out);
      if (kk == 16) k_irs_scan_i<16, float><<<g, 256, 0, s>>>(b, tb, bb, out);
      return;
    }
  }
  if (variant == 1 && sm <= 200 * 1024) {
    const long long grid = 5 * ((lines + LT - 1) / LT);
    k_irs_smem<T, TC, D, LT><<<(unsigned)grid, LT, sm, s>>>(b, tb, bb);
  } else {
    if (5 * lines >= 150000)  // about 8 warps per scheduler: the sweep is bound by the FP64 rate
      k_irs<T, TC, D, true><<<LAUNCH_N(5 * lines), 0, s>>>(b, tb, bb);
    else
      k_irs<T, TC, D><<<LAUNCH_N(5 * lines), 0, s>>>(b, tb, bb);
  }
}

template <typename T>
long long irs_lines_h(const DevBlock<T>& b, int D) {
  return D == 0 ? (long long)b.ny * b.nz : (D == 1 ? (long long)b.nx * b.nz : (long long)b.nx * b.ny);
}

template <typename T, typename TC>
void launch_irs_part_t(int part, const DevBlock<T>& b, const PhysParams& P, const IrsTables* tab, cudaStream_t s,
                       const int* variant, const StageArgs* A) {
  StageArgs Au;  // the update's stage (steady without one: lam = 1)
  memset(&Au, 0, sizeof(Au));
  if (A) Au = *A;
  const TC bb = (TC)(-P.smoo);
  const long long ncell = (long long)b.nx * b.ny * b.nz;
  if (P.irs_kind == 1) {  // psmoo + progon3: one thread per line
    if (part == 0) k_psmoo_line<T, TC, 0><<<LAUNCH_N(irs_lines_h(b, 0)), 0, s>>>(b);
    if (part == 1) k_psmoo_line<T, TC, 1><<<LAUNCH_N(irs_lines_h(b, 1)), 0, s>>>(b);
    if (part == 2) {
      k_psmoo_line<T, TC, 2><<<LAUNCH_N(irs_lines_h(b, 2)), 0, s>>>(b);
      k_update<T><<<LAUNCH_N(ncell), 0, s>>>(b, P, Au);
    }
    return;
  }
  if constexpr (std::is_same<T, double>::value && std::is_same<TC, float>::value) {
    // FP32 sweeps on FP64 storage: one FP32 copy through the three sweeps
    float* cp = (float*)b.F;
    if (part == 0) {
      // the tuned form of the i sweep: global-memory lines or shared-memory tiles
      constexpr int LT = 64;
      const size_t sm = irs_smem_bytes<float, LT>((b.il - 1) | 1);
      const int kk = irs_scan_k(b.il - 1);
      const long long nthr = 32 * 5 * irs_lines_h(b, 0);
      if (variant && variant[0] == 2 && kk) {
        const unsigned g = (unsigned)nblk(nthr, 256);
        if (kk == 2) k_irs_scan_i<2><<<g, 256, 0, s>>>(b, tab[0], bb, cp);
        if (kk == 4) k_irs_scan_i<4><<<g, 256, 0, s>>>(b, tab[0], bb, cp);
        if (kk == 6) k_irs_scan_i<6><<<g, 256, 0, s>>>(b, tab[0], bb, cp);
        if (kk == 8) k_irs_scan_i<8><<<g, 256, 0, s>>>(b, tab[0], bb, cp);
        if (kk == 12) k_irs_scan_i<12><<<g, 256, 0, s>>>(b, tab[0], bb, cp);
        if (kk == 16) k_irs_scan_i<16><<<g, 256, 0, s>>>(b, tab[0], bb, cp);
      } else if (variant && variant[0] == 1 && sm <= 200 * 1024)
        k_irs_smem_fill<LT><<<(unsigned)(5 * ((irs_lines_h(b, 0) + LT - 1) / LT)), LT, sm, s>>>(b, tab[0], bb, cp);
      else
        k_irs_mixed<double, float, 0><<<LAUNCH_N(5 * irs_lines_h(b, 0)), 0, s>>>(b, tab[0], bb, b.dw, cp, cp);
    }
    if (part == 1)
      k_irs_mixed<float, float, 1><<<LAUNCH_N(5 * irs_lines_h(b, 1)), 0, s>>>(b, tab[1], bb, cp, cp, cp);
    if (part == 2) {
      k_irs_mixed<float, double, 2><<<LAUNCH_N(5 * irs_lines_h(b, 2)), 0, s>>>(b, tab[2], bb, cp, cp, b.dw);
      k_update<T><<<LAUNCH_N(ncell), 0, s>>>(b, P, Au);
    }
    return;
  }
  if (part == 0) launch_irs_dir<T, TC, 0>(b, tab[0], bb, s, variant ? variant[0] : 0);
  if (part == 1) launch_irs_dir<T, TC, 1>(b, tab[1], bb, s, variant ? variant[1] : 0);
  if (part == 2) {
    launch_irs_dir<T, TC, 2>(b, tab[2], bb, s, variant ? variant[2] : 0);
    k_update<T><<<LAUNCH_N(ncell), 0, s>>>(b, P, Au);
  }
}

template <typename T>
void launch_irs_part(int part, const DevBlock<T>& b, const PhysParams& P, const IrsTables* tab, cudaStream_t s,
                     bool aux32, const int* variant, const StageArgs* A) {
  if (aux32)
    launch_irs_part_t<T, float>(part, b, P, tab, s, variant, A);
  else
    launch_irs_part_t<T, T>(part, b, P, tab, s, variant, A);
}

template <typename T>
void launch_irs(const DevBlock<T>& b, const PhysParams& P, const IrsTables* tab, cudaStream_t s, bool aux32,
                const int* variant, const StageArgs* A) {
  for (int part = 0; part < 3; part++) launch_irs_part<T>(part, b, P, tab, s, aux32, variant, A);
}

template <typename T>
void launch_cutcell(const DevBlock<T>& b, const PhysParams& P, unsigned* err, cudaStream_t s) {
  if (b.nmir > 0) k_cutcell<T><<<LAUNCH_N(b.nmir), 0, s>>>(b, P, err);
}

template <typename T>
void launch_bcond(const DevBlock<T>& b, const PhysParams& P, cudaStream_t s) {
  const long long n = 2LL * ((long long)(b.jb + 1) * (b.kb + 1) + (long long)(b.ib + 1) * (b.kb + 1) +
                             (long long)(b.ib + 1) * (b.jb + 1));
  const int tpb = tpb_for(n);
  // Six launches (three face passes, three corner phases) measured a little
  // faster inside the cycle graphs than one cooperative launch with grid
  // barriers; MGE_BCOND_COOP=1 selects the cooperative form (when every block
  // it needs fits on the device at once; residency per block size).
  static int resident[64][4] = {};
  static int coop_env = -1;
  if (coop_env < 0) {
    const char* e = getenv("MGE_BCOND_COOP");
    coop_env = (e && atoi(e) == 1) ? 1 : 0;
  }
  const int ti = tpb == 32 ? 0 : (tpb == 64 ? 1 : (tpb == 128 ? 2 : 3));
  int dev = 0;
  cudaGetDevice(&dev);
  if (coop_env && dev >= 0 && dev < 64 && resident[dev][ti] == 0) {
    int nsm = 0, per = 0, coop = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_bcond_coop<T>, tpb, 0);
    resident[dev][ti] = (coop && per > 0) ? nsm * per : -1;
  }
  const int grid = (coop_env && dev >= 0 && dev < 64) ? resident[dev][ti] : -1;
  if (grid > 0) {
    const int need = (int)std::max<long long>(1, std::min<long long>(nblk(n, tpb), grid));
    DevBlock<T> bb = b;
    PhysParams pp = P;
    void* args[] = {&bb, &pp};
    if (cudaLaunchCooperativeKernel((void*)k_bcond_coop<T>, need, tpb, args, 0, s) == cudaSuccess) return;
    cudaGetLastError();
  }
  for (int pass = 0; pass < 3; pass++) k_bc_pass<T><<<LAUNCH_N(n), 0, s>>>(b, P, pass);
  const long long nc = 4LL * (b.ib + b.jl + b.kl + 2);  // covers the items of phases 0 and 1
  for (int phase = 0; phase < 3; phase++) k_bc_corner<T><<<LAUNCH_N(phase == 2 ? 8 : nc), 0, s>>>(b, P, phase);
}

template <typename T>
void launch_rtrms(const DevBlock<T>& b, const PhysParams& P, int vt, double* partial, int npartial, double* out,
                  cudaStream_t s, unsigned* err) {
  k_rtrms_partial<T><<<npartial, RT_THREADS, 0, s>>>(b, P.cfl, vt, partial, npartial);
  k_rtrms_final<<<1, 32, 0, s>>>(partial, npartial, (double)b.nx * b.ny * b.nz, out, err);
}

template <typename TS, typename TD>
__global__ void k_convert(const TS* __restrict__ a, TD* __restrict__ b, long long n) {
  long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) b[q] = (TD)a[q];
}

void launch_convert(const void* src, bool src32, void* dst, bool dst32, long long n, cudaStream_t s) {
  if (n <= 0) return;
  if (src32 && !dst32) k_convert<float, double><<<nblk(n, TPB), TPB, 0, s>>>((const float*)src, (double*)dst, n);
  else if (!src32 && dst32) k_convert<double, float><<<nblk(n, TPB), TPB, 0, s>>>((const double*)src, (float*)dst, n);
  else if (src32) k_convert<float, float><<<nblk(n, TPB), TPB, 0, s>>>((const float*)src, (float*)dst, n);
  else k_convert<double, double><<<nblk(n, TPB), TPB, 0, s>>>((const double*)src, (double*)dst, n);
}

// movsurf.f90:31 (pnew = psurf + disp) and the wall velocity of
// bc_cutcell.f90:50 (qb = vel/vel_fs), one thread per record component
__global__ void k_movsurf(long long n3, const double* psurf, double* pnew, double* qb, double vel_fs) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  pnew[t] = psurf[t] + pnew[t];
  qb[t] = qb[t] / vel_fs;
}

void launch_movsurf(long long nmir, const double* psurf, double* pnew, double* qb, double vel_fs, cudaStream_t s) {
  if (nmir <= 0) return;
  k_movsurf<<<nblk(3 * nmir, TPB), TPB, 0, s>>>(3 * nmir, psurf, pnew, qb, vel_fs);
}

// opt-in shared memory of the tiled line sweeps; called once per device at set-up
void init_kernel_attributes() {
#define MGE_SMEM_ATTR(T, TC)                                                                                     \
  cudaFuncSetAttribute(k_irs_smem<T, TC, 0, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);     \
  cudaFuncSetAttribute(k_irs_smem<T, TC, 1, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);     \
  cudaFuncSetAttribute(k_irs_smem<T, TC, 2, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  MGE_SMEM_ATTR(double, double)
  MGE_SMEM_ATTR(double, float)
  MGE_SMEM_ATTR(float, float)
#undef MGE_SMEM_ATTR
  cudaFuncSetAttribute(k_irs_smem_fill<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

// grid of the cooperative kernel: every block resident at once
template <typename T, typename TA>
int coop_grid(int device) {
  static int cached[64] = {0};
  if (device < 0 || device >= 64) return 0;
  if (cached[device]) return cached[device];
  int nsm = 0, per = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_euler_coop<T, TA>, 256, 0);
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
  cached[device] = (coop && per > 0) ? nsm * per : -1;
  return cached[device];
}

template <typename T>
int launch_euler_coop(const DevBlock<T>& b, const PhysParams& P, const EulerLaunch& L, int device, cudaStream_t s,
                      bool aux32) {
  int grid = aux32 ? coop_grid<T, float>(device) : coop_grid<T, T>(device);
  if (grid <= 0) return -1;
  long long work = (long long)(b.ie) * b.je * b.ke;
  static int nsm = 0;
  if (!nsm && cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) nsm = 1;
  // at least one block per SM: the kernel deals items round-robin over the blocks
  int need = (int)std::min<long long>(std::max<long long>((work + 255) / 256, nsm), (long long)grid);
  if (L.max_ctas > 0 && need > L.max_ctas) need = L.max_ctas;
  if (need < 1) need = 1;
  EulerArgs E;
  memset(&E, 0, sizeof(E));
  E.mstage = L.mstage;
  E.do_timestep = L.do_timestep;
  E.lfir = L.lfir;
  E.lres = L.lres;
  E.rt = L.rt;
  for (int m = 0; m < L.mstage && m < 8; m++) E.st[m] = L.st[m];
  for (int d = 0; d < 3; d++) E.tab[d] = L.tab[d];
  E.rt_partial = L.rt_partial;
  E.npart = L.npart;
  E.rt_out = L.rt_out;
  E.err = L.err;
  E.trace = L.trace;
  DevBlock<T> bb = b;
  PhysParams pp = P;
  void* args[] = {&bb, &pp, &E};
  void* fn = aux32 ? (void*)k_euler_coop<T, float> : (void*)k_euler_coop<T, T>;
  cudaError_t e = cudaLaunchCooperativeKernel(fn, need, 256, args, 0, s);
  return e == cudaSuccess ? 0 : -2;
}

template <typename T>
void launch_depvars_all(const DevBlock<T>& b, const PhysParams& P, cudaStream_t s) {
  k_depvars_all<T><<<nblk(b.N, TPB), TPB, 0, s>>>(b, P.gamma);
}

template <typename T>
void launch_copy_ws(const DevBlock<T>& b, cudaStream_t s) {
  k_copy5<T><<<nblk(5 * b.N, TPB), TPB, 0, s>>>(b.w, b.ws, 5 * b.N);
}

template <typename T>
void launch_save_wn(const DevBlock<T>& b, cudaStream_t s) {
  k_save_wn<T><<<nblk(b.N, TPB), TPB, 0, s>>>(b);
}

template <typename T>
void launch_copy_wn(const DevBlock<T>& b, cudaStream_t s) {
  k_copy_wn<T><<<nblk(b.N, TPB), TPB, 0, s>>>(b);
}

template <typename T>
void launch_init_free(const DevBlock<T>& b, const PhysParams& P, cudaStream_t s) {
  k_init_free<T><<<nblk(b.N, TPB), TPB, 0, s>>>(b, P);
}

// a transfer's ratio and offset; an exact reciprocal of a power-of-two ratio
inline Xfer make_xfer(const int ratio[3], const int offset[3]) {
  Xfer X;
  for (int d = 0; d < 3; d++) {
    X.r[d] = ratio[d];
    X.o[d] = offset[d];
    X.rinv[d] = (ratio[d] > 0 && (ratio[d] & (ratio[d] - 1)) == 0) ? 1.0 / (double)ratio[d] : 0.0;
  }
  return X;
}

template <typename TC, typename TF>
void launch_collc(const DevBlock<TC>& c, const DevBlock<TF>& f, const int ratio[3], const int offset[3],
                  uint8_t* marker_c, cudaStream_t s) {
  Xfer X = make_xfer(ratio, offset);
  long long n = (long long)(f.nx / ratio[0]) * (f.ny / ratio[1]) * (f.nz / ratio[2]);
  k_collc<TC, TF><<<LAUNCH_N(n), 0, s>>>(c, f, X, marker_c);
}

template <typename TF, typename TC>
void launch_addw(const DevBlock<TF>& f, const DevBlock<TC>& c, const int ratio[3], const int offset[3], int fmg,
                 double* scratch, cudaStream_t s) {
  Xfer X = make_xfer(ratio, offset);
  long long n = (long long)f.nx * f.ny * f.nz;
  // the coarse corrections go to the stage scratch (at least 64 fields of
  // the largest block), free between euler calls
  if (!fmg) k_addw_diff<TC><<<LAUNCH_N(c.N), 0, s>>>(c, scratch);
  k_addw<TF, TC><<<LAUNCH_N(n), 0, s>>>(f, c, X, fmg, scratch);
}

template <typename TF, typename TC>
void launch_embed(const DevBlock<TF>& f, const DevBlock<TC>& c, const int ratio[3], const int offset[3],
                  const PhysParams& P, cudaStream_t s) {
  Xfer X = make_xfer(ratio, offset);
  k_embed<TF, TC><<<LAUNCH_N(f.N), 0, s>>>(f, c, X, P.gamma);
}

template <typename T>
void launch_overlap(const DevBlock<T>& g, const DevBlock<T>& p, const long long* dst, const long long* src,
                    const double* fac, long long n, const PhysParams& P, cudaStream_t s) {
  if (n > 0) k_overlap<T><<<LAUNCH_N(n), 0, s>>>(g, p, dst, src, fac, n, P.gamma);
}

template <typename T>
void launch_forces(const DevBlock<T>& b, const double* origin, const double* h, const double* center, double mu,
                   double* out7, cudaStream_t s) {
  k_forces<T><<<1, 256, 0, s>>>(b, origin[0], origin[1], origin[2], h[0], h[1], h[2], center[0], center[1], center[2],
                                mu, out7);
}

// --------------------------------------------------------------- a group's lockstep steps
size_t xfer_size() { return sizeof(Xfer); }
void make_xfer_host(const int ratio[3], const int offset[3], void* out) {
  Xfer X = make_xfer(ratio, offset);
  memcpy(out, &X, sizeof(Xfer));
}

template <typename T, typename F>
static void go_multi(const MultiLevel& L, MultiArgs<T>& M, int kind, F f, cudaStream_t s) {
  if (L.tot[kind] <= 0) return;
  M.off = L.off[kind];
  k_multi<T, F><<<(unsigned)(L.tot[kind] / 256), 256, 0, s>>>(M, f);
}

template <typename T>
static MultiArgs<T> multi_args(const MultiLevel& L) {
  return MultiArgs<T>{(const DevBlock<T>*)L.B, L.P, L.err, L.tab, L.rt_partial, L.npart, L.rt_out, nullptr, L.nc};
}

template <typename T>
static void multi_bcond(const MultiLevel& L, MultiArgs<T>& M, cudaStream_t s) {
  for (int pass = 0; pass < 3; pass++) go_multi(L, M, MK_BC, FBcPass<T>{pass}, s);
  go_multi(L, M, MK_CORNER0, FCorner<T>{0}, s);
  go_multi(L, M, MK_CORNER1, FCorner<T>{1}, s);
  go_multi(L, M, MK_CORNER2, FCorner<T>{2}, s);
}

// timestep (optionally) and euler.f90:1-462 on one block of every case: the
// phases of enqueue_euler's per-phase path (line sweeps in global memory)
template <typename T>
static void multi_euler_t(const MultiLevel& L, const StageArgs* A, int mstage, bool with_timestep, bool lfir,
                          bool rt, cudaStream_t s) {
  MultiArgs<T> M = multi_args<T>(L);
  if (with_timestep) {
    go_multi(L, M, MK_ONE, FDtimReset<T>{}, s);
    if (L.aux32)
      go_multi(L, M, MK_PHYS, FTimestep<T, float>{}, s);
    else
      go_multi(L, M, MK_PHYS, FTimestep<T, T>{}, s);
  }
  if (lfir) go_multi(L, M, MK_N5, FCopyWs<T>{}, s);
  go_multi(L, M, MK_N, FSaveWn<T>{}, s);
  for (int m = 1; m <= mstage; m++) {
    const StageArgs& a = A[m - 1];
    if (L.fast) {
      go_multi(L, M, MK_PREP, FPrep<T, true>{a.dissip_on}, s);
      if (a.dissip_on) go_multi(L, M, MK_FACE, FFaceDiss<T>{(T)a.cd}, s);
    } else {
      go_multi(L, M, MK_PREP, FPrep<T, false>{a.dissip_on}, s);
      if (a.dissip_on)
        go_multi(L, M, MK_FACE, FFace<T>{a.dissip_on, (T)a.cd}, s);
      else
        go_multi(L, M, MK_FACE, FFaceConv<T>{}, s);
    }
    go_multi(L, M, MK_REC, FRec<T>{a.dissip_on, (T)a.cd}, s);
    if (L.fast)
      go_multi(L, M, MK_PHYS, FCombine<T, true>{a}, s);
    else
      go_multi(L, M, MK_PHYS, FCombine<T, false>{a}, s);
    if (a.lres) return;
    if (a.irs) {
      if constexpr (std::is_same<T, double>::value) {
        if (L.aux32) {
          go_multi(L, M, MK_IRS0, FIrsMixed<double, float, 0>{}, s);
          go_multi(L, M, MK_IRS1, FIrsMixed<float, float, 1>{}, s);
          go_multi(L, M, MK_IRS2, FIrsMixed<float, double, 2>{}, s);
        } else {
          go_multi(L, M, MK_IRS0, FIrs<T, T, 0>{}, s);
          go_multi(L, M, MK_IRS1, FIrs<T, T, 1>{}, s);
          go_multi(L, M, MK_IRS2, FIrs<T, T, 2>{}, s);
        }
      } else {
        go_multi(L, M, MK_IRS0, FIrs<T, T, 0>{}, s);
        go_multi(L, M, MK_IRS1, FIrs<T, T, 1>{}, s);
        go_multi(L, M, MK_IRS2, FIrs<T, T, 2>{}, s);
      }
      go_multi(L, M, MK_PHYS, FUpdate<T>{a}, s);
    }
    go_multi(L, M, MK_REC, FCutcell<T>{}, s);
    multi_bcond(L, M, s);
  }
  if (rt) {
    go_multi(L, M, MK_RTP, FRtrmsPartial<T>{}, s);
    go_multi(L, M, MK_ONE, FRtrmsFinal<T>{}, s);
  }
}

// every case's residual of the cycle and its error word, into two arrays
template <typename T> struct FGather {
  double* res;
  unsigned* errs;
  __device__ void operator()(const MultiArgs<T>& M, int q, long long t) const {
    if (t == 0) {
      res[q] = *M.rt_out[q];
      errs[q] = *M.err[q];
    }
  }
};

void gather_residuals(const MultiLevel& L, double* res, unsigned* errs, cudaStream_t s) {
  if (L.f32) {
    MultiArgs<float> M = multi_args<float>(L);
    go_multi(L, M, MK_ONE, FGather<float>{res, errs}, s);
  } else {
    MultiArgs<double> M = multi_args<double>(L);
    go_multi(L, M, MK_ONE, FGather<double>{res, errs}, s);
  }
}

// The whole update of every case of a group as ONE persistent cooperative
// launch: the phases of multi_euler_t in the same order, a grid-wide barrier
// between dependent phases, each phase's thread blocks of 256 items dealt
// over the resident blocks (a block serves one case at a time, so the
// per-block reductions stay within a case).  For the small levels, where a
// phase's launch costs more than its work.
struct GroupEuler {
  const long long* off[MK_COUNT];
  long long tot[MK_COUNT];
  int mstage, do_timestep, lfir, rt, fast, aux32;
  StageArgs st[8];  // the stages (at most 8)
};

__device__ __forceinline__ int case_of(const long long* off, int nc, long long base) {
  int lo = 0, hi = nc - 1;  // the last q with off[q] <= base
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= base) lo = mid; else hi = mid - 1;
  }
  return lo;
}

template <typename T, typename F>
__device__ __forceinline__ void group_phase(const MultiArgs<T>& M, const GroupEuler& G, int kind, const F& f) {
  const long long tot = G.tot[kind];
  for (long long base = (long long)blockIdx.x * 256; base < tot; base += (long long)gridDim.x * 256) {
    const int q = case_of(G.off[kind], M.nc, base);
    f(M, q, base - G.off[kind][q] + threadIdx.x);
  }
}

template <typename T, typename TA>
__global__ void __launch_bounds__(256, 1) k_group_euler(MultiArgs<T> M, GroupEuler G) {
  cg::grid_group grid = cg::this_grid();
  if (G.do_timestep) {
    group_phase(M, G, MK_ONE, FDtimReset<T>{});
    grid.sync();
    group_phase(M, G, MK_PHYS, FTimestep<T, TA>{});
  }
  if (G.lfir) group_phase(M, G, MK_N5, FCopyWs<T>{});
  group_phase(M, G, MK_N, FSaveWn<T>{});
  grid.sync();
  for (int m = 1; m <= G.mstage; m++) {
    const StageArgs& a = G.st[m - 1];
    if (G.fast) {
      group_phase(M, G, MK_PREP, FPrep<T, true>{a.dissip_on});
      grid.sync();
      if (a.dissip_on) group_phase(M, G, MK_FACE, FFaceDiss<T>{(T)a.cd});
    } else {
      group_phase(M, G, MK_PREP, FPrep<T, false>{a.dissip_on});
      grid.sync();
      if (a.dissip_on)
        group_phase(M, G, MK_FACE, FFace<T>{a.dissip_on, (T)a.cd});
      else
        group_phase(M, G, MK_FACE, FFaceConv<T>{});
    }
    group_phase(M, G, MK_REC, FRec<T>{a.dissip_on, (T)a.cd});
    grid.sync();
    if (G.fast)
      group_phase(M, G, MK_PHYS, FCombine<T, true>{a});
    else
      group_phase(M, G, MK_PHYS, FCombine<T, false>{a});
    grid.sync();
    if (a.lres) return;
    if (a.irs) {
      if constexpr (std::is_same<T, double>::value && std::is_same<TA, float>::value) {
        group_phase(M, G, MK_IRS0, FIrsMixed<double, float, 0>{});
        grid.sync();
        group_phase(M, G, MK_IRS1, FIrsMixed<float, float, 1>{});
        grid.sync();
        group_phase(M, G, MK_IRS2, FIrsMixed<float, double, 2>{});
      } else {
        group_phase(M, G, MK_IRS0, FIrs<T, T, 0>{});
        grid.sync();
        group_phase(M, G, MK_IRS1, FIrs<T, T, 1>{});
        grid.sync();
        group_phase(M, G, MK_IRS2, FIrs<T, T, 2>{});
      }
      grid.sync();
      group_phase(M, G, MK_PHYS, FUpdate<T>{a});
      grid.sync();
    }
    group_phase(M, G, MK_REC, FCutcell<T>{});
    grid.sync();
    for (int pass = 0; pass < 3; pass++) {
      group_phase(M, G, MK_BC, FBcPass<T>{pass});
      grid.sync();
    }
    for (int phase = 0; phase < 3; phase++) {
      group_phase(M, G, MK_CORNER0 + phase, FCorner<T>{phase});
      grid.sync();
    }
  }
  if (G.rt) {
    group_phase(M, G, MK_RTP, FRtrmsPartial<T>{});
    grid.sync();
    group_phase(M, G, MK_ONE, FRtrmsFinal<T>{});
  }
}

// resident blocks of the group kernel on the device (0: no cooperative launch)
template <typename T, typename TA>
static int group_grid() {
  static int cached[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return 0;
  if (cached[dev]) return cached[dev] > 0 ? cached[dev] : 0;
  int nsm = 0, per = 0, coop = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_group_euler<T, TA>, 256, 0);
  cached[dev] = (coop && per > 0) ? nsm * per : -1;
  return cached[dev] > 0 ? cached[dev] : 0;
}

// the group's update as one cooperative launch; false when it cannot run so
template <typename T>
static bool group_euler_coop(const MultiLevel& L, const StageArgs* A, int mstage, bool with_timestep, bool lfir,
                             bool rt, cudaStream_t s) {
  const bool mixed32 = std::is_same<T, double>::value && L.aux32;
  const int gmax = mixed32 ? group_grid<T, float>() : group_grid<T, T>();
  if (gmax <= 0) return false;
  GroupEuler G;
  memset(&G, 0, sizeof(G));
  long long most = 0;
  for (int k = 0; k < MK_COUNT; k++) {
    G.off[k] = L.off[k];
    G.tot[k] = L.tot[k];
    most = std::max(most, L.tot[k] / 256);
  }
  G.mstage = mstage;
  G.do_timestep = with_timestep;
  G.lfir = lfir;
  G.rt = rt;
  G.fast = L.fast;
  G.aux32 = L.aux32;
  for (int m = 0; m < mstage && m < 8; m++) G.st[m] = A[m];
  MultiArgs<T> M = multi_args<T>(L);
  const int grid = (int)std::max<long long>(1, std::min<long long>(most, gmax));
  void* args[] = {&M, &G};
  void* fn = mixed32 ? (void*)k_group_euler<T, float> : (void*)k_group_euler<T, T>;
  if (cudaLaunchCooperativeKernel(fn, grid, 256, args, 0, s) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return true;
}

void multi_euler(const MultiLevel& L, const StageArgs* A, int mstage, bool with_timestep, bool lfir, bool rt,
                 cudaStream_t s) {
  if (L.coop) {
    const bool done = L.f32 ? group_euler_coop<float>(L, A, mstage, with_timestep, lfir, rt, s)
                            : group_euler_coop<double>(L, A, mstage, with_timestep, lfir, rt, s);
    if (done) return;
  }
  if (L.f32)
    multi_euler_t<float>(L, A, mstage, with_timestep, lfir, rt, s);
  else
    multi_euler_t<double>(L, A, mstage, with_timestep, lfir, rt, s);
}

template <typename TC, typename TF, typename F>
static void go_pair(const MultiPair& Pp, MultiPairArgs<TC, TF>& M, int kind, F f, cudaStream_t s) {
  if (Pp.tot[kind] <= 0) return;
  M.off = Pp.off[kind];
  k_multi2<TC, TF, F><<<(unsigned)(Pp.tot[kind] / 256), 256, 0, s>>>(M, f);
}

template <typename TC, typename TF>
static MultiPairArgs<TC, TF> pair_args(const MultiPair& Pp) {
  return MultiPairArgs<TC, TF>{(const DevBlock<TC>*)Pp.C, (const DevBlock<TF>*)Pp.F, (const Xfer*)Pp.X, Pp.marker,
                               Pp.dc, Pp.P, nullptr, Pp.nc};
}

// the pair's precisions: (coarse, fine) in {(double, double), (float, double), (float, float)}
template <typename Fn>
static void with_pair_types(const MultiPair& Pp, Fn&& fn) {
  if (!Pp.c32 && !Pp.f32)
    fn((double*)nullptr, (double*)nullptr);
  else if (Pp.c32 && !Pp.f32)
    fn((float*)nullptr, (double*)nullptr);
  else
    fn((float*)nullptr, (float*)nullptr);
}

// movco.f90:21-47 for the group: restriction of each case's child onto its
// block on this level, depvars, wn, bcond (one block per level: no overlap)
void multi_movco_level(const MultiLevel& L, const MultiPair* pair, cudaStream_t s) {
  if (pair)
    with_pair_types(*pair, [&](auto* tc, auto* tf) {
      using TC = std::remove_pointer_t<decltype(tc)>;
      using TF = std::remove_pointer_t<decltype(tf)>;
      MultiPairArgs<TC, TF> M = pair_args<TC, TF>(*pair);
      go_pair(*pair, M, MP_CN, FMarkerClear<TC, TF>{}, s);
      go_pair(*pair, M, MP_COLLC, FCollc<TC, TF>{}, s);
    });
  auto rest = [&](auto* tp) {
    using T = std::remove_pointer_t<decltype(tp)>;
    MultiArgs<T> M = multi_args<T>(L);
    go_multi(L, M, MK_N, FDepvars<T>{}, s);
    go_multi(L, M, MK_N, FCopyWn<T>{}, s);
    multi_bcond(L, M, s);
  };
  if (L.f32)
    rest((float*)nullptr);
  else
    rest((double*)nullptr);
}

// movfin.f90:20-39 for the group: prolongation from each case's parent,
// depvars, bc_embed, bcond
void multi_movfin_level(const MultiLevel& L, const MultiPair& pair, bool fmg, cudaStream_t s) {
  with_pair_types(pair, [&](auto* tc, auto* tf) {
    using TC = std::remove_pointer_t<decltype(tc)>;
    using TF = std::remove_pointer_t<decltype(tf)>;
    MultiPairArgs<TC, TF> M = pair_args<TC, TF>(pair);
    if (!fmg) go_pair(pair, M, MP_CN, FAddwDiff<TC, TF>{}, s);
    go_pair(pair, M, MP_FPHYS, FAddw<TC, TF>{fmg ? 1 : 0}, s);
    MultiArgs<TF> F = multi_args<TF>(L);
    go_multi(L, F, MK_N, FDepvars<TF>{}, s);
    go_pair(pair, M, MP_FN, FEmbed<TC, TF>{}, s);
    multi_bcond(L, F, s);
  });
}

// explicit instantiations
#define MGE_INST(T)                                                                                              \
  template void launch_timestep<T>(const DevBlock<T>&, const PhysParams&, unsigned*, cudaStream_t, bool);       \
  template void launch_solut<T>(const DevBlock<T>&, const PhysParams&, double, double, int, double*, cudaStream_t); \
  template void launch_stage<T>(const DevBlock<T>&, const PhysParams&, const StageArgs&, unsigned*, cudaStream_t,     \
                                cudaStream_t, cudaEvent_t, cudaEvent_t);                                               \
  template void launch_stage_part<T>(int, const DevBlock<T>&, const PhysParams&, const StageArgs&, unsigned*,       \
                                     cudaStream_t);                                                             \
  template void launch_irs_part<T>(int, const DevBlock<T>&, const PhysParams&, const IrsTables*, cudaStream_t,    \
                                   bool, const int*, const StageArgs*);                                         \
  template int launch_euler_coop<T>(const DevBlock<T>&, const PhysParams&, const EulerLaunch&, int, cudaStream_t,  \
                                    bool);                                                                      \
  template void launch_irs<T>(const DevBlock<T>&, const PhysParams&, const IrsTables*, cudaStream_t, bool,       \
                              const int*, const StageArgs*);                                                    \
  template void launch_cutcell<T>(const DevBlock<T>&, const PhysParams&, unsigned*, cudaStream_t);              \
  template void launch_bcond<T>(const DevBlock<T>&, const PhysParams&, cudaStream_t);                           \
  template void launch_rtrms<T>(const DevBlock<T>&, const PhysParams&, int, double*, int, double*, cudaStream_t, \
                                unsigned*);                                                                    \
  template void launch_depvars_all<T>(const DevBlock<T>&, const PhysParams&, cudaStream_t);                     \
  template void launch_copy_ws<T>(const DevBlock<T>&, cudaStream_t);                                            \
  template void launch_save_wn<T>(const DevBlock<T>&, cudaStream_t);                                            \
  template void launch_copy_wn<T>(const DevBlock<T>&, cudaStream_t);                                            \
  template void launch_init_free<T>(const DevBlock<T>&, const PhysParams&, cudaStream_t);                       \
  template void launch_forces<T>(const DevBlock<T>&, const double*, const double*, const double*, double, double*,  \
                                 cudaStream_t);                                                                  \
  template void launch_overlap<T>(const DevBlock<T>&, const DevBlock<T>&, const long long*, const long long*,        \
                                  const double*, long long, const PhysParams&, cudaStream_t);
MGE_INST(double)
MGE_INST(float)
#undef MGE_INST
#define MGE_XFER(TC, TF)                                                                                         \
  template void launch_collc<TC, TF>(const DevBlock<TC>&, const DevBlock<TF>&, const int*, const int*, uint8_t*,   \
                                     cudaStream_t);                                                             \
  template void launch_addw<TF, TC>(const DevBlock<TF>&, const DevBlock<TC>&, const int*, const int*, int,          \
                                    double*, cudaStream_t);                                                     \
  template void launch_embed<TF, TC>(const DevBlock<TF>&, const DevBlock<TC>&, const int*, const int*,              \
                                     const PhysParams&, cudaStream_t);
MGE_XFER(double, double)
MGE_XFER(float, double)
MGE_XFER(float, float)
#undef MGE_XFER


}  // namespace mge
