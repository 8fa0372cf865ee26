// mge_runtime.cu -- host runtime and C-ABI of the GB300 multigrid cycle.
//
// One mge_ctx owns a case: its level hierarchy of uniform blocks, every field
// resident in device memory for the whole solve, one CUDA stream, and the
// CUDA graphs of the multigrid cycle.  The entry points of include/mge_gpu.h
// replace the reference's calls one for one (timestep.f90, euler.f90,
// movco.f90, movfin.f90, solver.f90); mge_solve runs solver.f90's FMG loop
// with each multigrid cycle captured once per FMG level and replayed.
#include <algorithm>
#include <atomic>
#include <type_traits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <string>
#include <vector>

#include "../../include/mge_gpu.h"
#include "mge_internal.h"

using namespace mge;

#define MGE_STR2(x) #x
#define MGE_STR(x) MGE_STR2(x)

namespace {

struct HRec {
  int ccid[3], scid[3], faceid, zz, npoint;
  int ijk[MGE_MAX_CLOUD][3];
  double coef[MGE_MAX_CLOUD], nvec[3], qb[3], area, psurf[3];
};

struct Block {
  int level = 0, serial = 0;
  int nx = 0, ny = 0, nz = 0, il = 0, jl = 0, kl = 0, ie = 0, je = 0, ke = 0, ib = 0, jb = 0, kb = 0;
  int Pi = 0, Pj = 0, Pk = 0;
  long long N = 0;
  double h[3] = {0, 0, 0}, origin[3] = {0, 0, 0}, vol = 0;
  double s[3] = {0, 0, 0};
  int bctype[6] = {0, 0, 0, 0, 0, 0};
  double fnv[6][3] = {};
  int parent = -1, ratio[3] = {1, 1, 1}, offset[3] = {0, 0, 0};
  std::vector<int32_t> blank_h;
  std::vector<HRec> recs;
  // same-level overlap (bc_overlap.f90:32-90): per partner block of the
  // level, the ghost cells of this block inside the partner's physical
  // cells, the partner's stencil base cell and the 8 trilinear weights
  struct Overlap {
    int partner = 0;  // serial
    long long n = 0;
    long long *dst = nullptr, *src = nullptr;
    double* fac = nullptr;
  };
  std::vector<Overlap> ovl;
  // device allocations; state fields hold doubles, or floats when f32
  bool f32 = false;    // FP32 storage and arithmetic (coarse levels of the mixed mode)
  bool aux32 = false;  // FP32 time step and smoothing on FP64 storage (finest level of the mixed mode)
  bool fast = false;   // the contracted FP64 residual (finest level of the mixed and refined forms)
  bool use_coop = false;   // run timestep + euler as one cooperative launch
  int irs_var[3] = {0, 0, 0};  // line-sweep variant per direction (autotuned)
  size_t esz = 8;
  void *w1 = nullptr, *w2 = nullptr;  // previous physical time steps (unsteady only)
  void *w = nullptr, *p = nullptr, *wn = nullptr, *ws = nullptr, *dw = nullptr, *fw = nullptr, *wr = nullptr,
       *qf = nullptr, *vdtim = nullptr, *lam = nullptr;
  void* eps = nullptr;  // 3N psmoo coefficients (irs_variant 1 only)
  double* dtim = nullptr;
  uint8_t *blank = nullptr, *marker = nullptr;
  int32_t* cutmap = nullptr;
  int32_t *rec_i = nullptr, *rec_cloud = nullptr, *tgt_off = nullptr, *tgt_ops = nullptr;
  double *rec_coef = nullptr, *rec_nvec = nullptr, *rec_qb = nullptr, *rec_area = nullptr;
  double *rec_psurf = nullptr, *rec_pnew = nullptr;  // [nmir][3] surface points, as given and as moved
  void *rec_wsol = nullptr, *rec_psol = nullptr, *rec_wall = nullptr;
  double* irs = nullptr;
  float* irs32 = nullptr;
  IrsTables tabs[3];
  double *rt_partial = nullptr, *rt_cur = nullptr, *forces = nullptr;
  int npart = 1;
  int m0 = 0;
  // every cloud cell of the records processed by bc_cutcell is physical, so
  // bc_cutcell (reads those cells, writes only the records) and bcond
  // (writes only ghost cells) touch disjoint data and may run concurrently
  bool cut_beside_bcond = false;
  std::vector<double> rtrms;  // host history rtrms(ncyc)
  DevBlock<double> dev;       // view when !f32
  DevBlock<float> dev32;      // view when f32
};

// run f on the block's typed view: f(DevBlock<double>&) or f(DevBlock<float>&)
template <typename F>
void with_dev(Block& b, F&& f) {
  if (b.f32)
    f(b.dev32);
  else
    f(b.dev);
}

}  // namespace

struct mge_ctx {
  mge_params prm;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;                 // record pass beside the face pass
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  std::vector<std::vector<Block>> lv;
  std::vector<std::pair<int, int>> order;  // (level, serial) in mge_add_block order
  int itime = 0;                           // physical time step counter (unsteady mode)
  std::string err;
  unsigned* d_err = nullptr;
  unsigned* h_err = nullptr;  // pinned
  double* h_rt = nullptr;     // pinned readback of residuals
  double* scratch = nullptr;
  size_t bytes = 0;
  PhysParams P;
  bool committed = false;
  std::vector<void*> allocs;
  std::vector<cudaGraphExec_t> graphs;  // one captured multigrid cycle per FMG level
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_cycle_ms = 0.0;
  std::vector<long long> graph_kernels;  // kernel nodes per captured cycle
  long long launches = 0;                // kernels launched through mge_cycle
  long long coop_max_cells = 300000;     // blocks up to this size run euler as one cooperative launch
  int coop_max_ctas = 0;                 // cap on the cooperative grid (0: all resident blocks)
  cudaEvent_t ev_done = nullptr;         // end of an asynchronous cycle
  bool autotune = true;                  // tune launch forms at init_flow
  bool tune_path = true;                 // ... including cooperative vs per-phase euler
  std::string plan;                      // fixed launch forms per level (MGE_TUNE_PLAN), instead of tuning
  int pending_mlvl = 0;                  // level of the cycle in flight (0: none)
  unsigned long long* coop_trace = nullptr;
  unsigned long long uid = 0;            // process-unique id (group plans key on it)
  unsigned gen = 0;                      // bumped whenever device fields move (precision switch)
  void* group_pending = nullptr;         // the group plan whose cycle this case is in
  cudaEvent_t ev_group = nullptr;        // this case's stream, ahead of a group cycle
};

namespace {

int fail(mge_ctx* c, int code, const std::string& m) {
  if (c) c->err = m;
  return code;
}

int cuda_fail(mge_ctx* c, cudaError_t e, const char* where) {
  return fail(c, MGE_ECUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(x)                                           \
  do {                                                  \
    cudaError_t e_ = (x);                               \
    if (e_ != cudaSuccess) return cuda_fail(c, e_, #x); \
  } while (0)

template <typename T>
int dalloc(mge_ctx* c, T** p, size_t n) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(c, MGE_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  c->allocs.push_back(q);
  c->bytes += std::max<size_t>(n, 1) * sizeof(T);
  *p = (T*)q;
  return MGE_OK;
}

Block* getb(mge_ctx* c, int level, int serial) {
  if (!c || level < 1 || level > (int)c->lv.size()) return nullptr;
  auto& L = c->lv[level - 1];
  if (serial < 1 || serial > (int)L.size()) return nullptr;
  return &L[serial - 1];
}

int check_err(mge_ctx* c) {
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "stream");
  e = cudaMemcpy(c->h_err, c->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(c, e, "error word");
  unsigned w = *c->h_err;
  if (w) {
    cudaMemset(c->d_err, 0, sizeof(unsigned));
    if (w & ERR_NEGPRESS) return fail(c, MGE_ENEGPRESS, "timestep: negative or NaN c^2 (timestep.f90:45-48)");
    if (w & ERR_ZERORHO) return fail(c, MGE_EZERORHO, "efluxb: zero density at a cut cell (efluxb.f90:61-64)");
    if (w & ERR_NAN) return fail(c, MGE_ENAN, "bc_cutcell: wsol is NaN (bc_cutcell.f90:147-156)");
    if (w & ERR_NANRES) return fail(c, MGE_ENAN, "NaN residual (solver.f90:180)");
  }
  return MGE_OK;
}

// ---------------------------------------------------------------- device ops
void enqueue_timestep(mge_ctx* c, Block& b) {
  with_dev(b, [&](auto& D) {
    using T = typename std::remove_reference_t<decltype(D)>::value_type;
    launch_timestep<T>(D, c->P, c->d_err, c->stream, b.aux32);
  });
}

StageArgs stage_args(const mge_params& P, int m, int mgl, int mlvl, bool lres, bool lfir, int itime) {
  StageArgs A;
  std::memset(&A, 0, sizeof(A));
  A.m = m;
  A.fn = P.cstp[m - 1] * P.cfl;
  A.cd = P.cdis[m - 1];
  A.dissip_on = P.cdis[m - 1] > 0.0;
  A.scale_fw = m > 1;
  A.forcing = mgl < mlvl;
  A.first_forcing = lfir && m == 1;
  A.lres = lres;
  A.irs = (m % 2 != 0) && P.smoo > 0.0 && !lres;
  A.vt = P.vt;
  // euler.f90:249-275: the transient source needs itime >= 1 (none in the first physical step)
  A.tmode = P.execmode == 1 ? (itime > 1 ? 2 : (itime == 1 ? 1 : 0)) : 0;
  return A;
}

// timestep.f90 (optionally) followed by euler.f90:1-462 on one block;
// nstage_limit > 0 stops after that stage (parity probes)
void enqueue_euler(mge_ctx* c, Block& b, int mgl, int mlvl, bool lres, bool lfir, int nstage_limit, bool rt,
                   bool with_timestep = false, int itime = -1) {
  const mge_params& P = c->prm;
  if (itime < 0) itime = c->itime;
  const int mstage = (nstage_limit > 0) ? std::min(P.mstage, nstage_limit) : P.mstage;
  const bool want_rt = rt && (nstage_limit <= 0 || nstage_limit >= P.mstage) && !lres;
  if (b.use_coop) {
    EulerLaunch L;
    std::memset(&L, 0, sizeof(L));
    L.mstage = mstage;
    L.do_timestep = with_timestep;
    L.lfir = lfir;
    L.lres = lres;
    L.rt = want_rt;
    for (int m = 1; m <= mstage; m++) {
      L.st[m - 1] = stage_args(P, m, mgl, mlvl, lres, lfir, itime);
      L.st[m - 1].fast = b.fast;
    }
    for (int d = 0; d < 3; d++) L.tab[d] = b.tabs[d];
    L.rt_partial = b.rt_partial;
    L.npart = b.npart;
    L.rt_out = b.rt_cur;
    L.err = c->d_err;
    L.trace = c->coop_trace;
    L.max_ctas = c->coop_max_ctas;
    int rc = -1;
    with_dev(b, [&](auto& D) {
      using T = typename std::remove_reference_t<decltype(D)>::value_type;
      rc = launch_euler_coop<T>(D, c->P, L, c->device, c->stream, b.aux32);
    });
    if (rc == 0) return;
    cudaGetLastError();  // cooperative launch unavailable: fall through to per-phase launches
  }
  // the time step (reads w, p; writes vdtim, lam, dtim) and the copies of w
  // into ws and wn touch disjoint outputs: the copies run beside it
  const bool copies_beside = with_timestep && c->side;
  if (copies_beside) {
    cudaEventRecord(c->ev_fork, c->stream);
    cudaStreamWaitEvent(c->side, c->ev_fork, 0);
    with_dev(b, [&](auto& D) {
      using T = typename std::remove_reference_t<decltype(D)>::value_type;
      if (lfir) launch_copy_ws<T>(D, c->side);
      launch_save_wn<T>(D, c->side);
    });
    cudaEventRecord(c->ev_join, c->side);
    enqueue_timestep(c, b);
    cudaStreamWaitEvent(c->stream, c->ev_join, 0);
  } else if (with_timestep) {
    enqueue_timestep(c, b);
  }
  with_dev(b, [&](auto& D) {
    using T = typename std::remove_reference_t<decltype(D)>::value_type;
    if (!copies_beside) {
      if (lfir) launch_copy_ws<T>(D, c->stream);
      launch_save_wn<T>(D, c->stream);
    }
    for (int m = 1; m <= mstage; m++) {
      StageArgs A = stage_args(P, m, mgl, mlvl, lres, lfir, itime);
      A.fast = b.fast;
      launch_stage<T>(D, c->P, A, c->d_err, c->stream, c->side, c->ev_fork, c->ev_join);
      if (lres) return;
      if (A.irs) launch_irs<T>(D, c->P, b.tabs, c->stream, b.aux32, b.irs_var, &A);
      if (b.cut_beside_bcond && c->side) {  // disjoint data: the record pass beside the boundary passes
        cudaEventRecord(c->ev_fork, c->stream);
        cudaStreamWaitEvent(c->side, c->ev_fork, 0);
        launch_cutcell<T>(D, c->P, c->d_err, c->side);
        cudaEventRecord(c->ev_join, c->side);
        launch_bcond<T>(D, c->P, c->stream);
        cudaStreamWaitEvent(c->stream, c->ev_join, 0);
      } else {
        launch_cutcell<T>(D, c->P, c->d_err, c->stream);
        launch_bcond<T>(D, c->P, c->stream);
      }
    }
    if (want_rt) launch_rtrms<T>(D, c->P, P.vt, b.rt_partial, b.npart, b.rt_cur, c->stream, c->d_err);
  });
}

// the restriction of one child onto its parent, in the pair's precisions
void enqueue_collc(mge_ctx* c, Block& b, Block& f) {
  with_dev(b, [&](auto& DC) {
    using TC = typename std::remove_reference_t<decltype(DC)>::value_type;
    with_dev(f, [&](auto& DF) {
      using TF = typename std::remove_reference_t<decltype(DF)>::value_type;
      if constexpr (sizeof(TC) <= sizeof(TF)) launch_collc<TC, TF>(DC, DF, f.ratio, f.offset, b.marker, c->stream);
    });
  });
}

void enqueue_addw_embed(mge_ctx* c, Block& f, Block& pb, bool fmg, bool embed) {
  with_dev(f, [&](auto& DF) {
    using TF = typename std::remove_reference_t<decltype(DF)>::value_type;
    with_dev(pb, [&](auto& DC) {
      using TC = typename std::remove_reference_t<decltype(DC)>::value_type;
      if constexpr (sizeof(TC) <= sizeof(TF)) {
        if (embed)
          launch_embed<TF, TC>(DF, DC, f.ratio, f.offset, c->P, c->stream);
        else
          launch_addw<TF, TC>(DF, DC, f.ratio, f.offset, fmg ? 1 : 0, c->scratch, c->stream);
      }
    });
  });
}

void enqueue_simple(mge_ctx* c, Block& b, int what) {
  with_dev(b, [&](auto& D) {
    using T = typename std::remove_reference_t<decltype(D)>::value_type;
    if (what == 0) launch_depvars_all<T>(D, c->P, c->stream);
    if (what == 1) launch_copy_wn<T>(D, c->stream);
    if (what == 2) launch_bcond<T>(D, c->P, c->stream);
    if (what == 3) launch_init_free<T>(D, c->P, c->stream);
    if (what == 4) launch_cutcell<T>(D, c->P, c->d_err, c->stream);
  });
}

// bc_overlap.f90:32-90 on level mgl: every block's ghost cells inside a
// partner's physical cells, partners in serial order (a later partner's
// value stands where two overlap)
void enqueue_overlap(mge_ctx* c, int mgl) {
  auto& L = c->lv[mgl - 1];
  for (Block& g : L)
    for (const Block::Overlap& o : g.ovl) {
      Block& p = L[o.partner - 1];
      with_dev(g, [&](auto& DG) {
        using T = typename std::remove_reference_t<decltype(DG)>::value_type;
        with_dev(p, [&](auto& DP) {
          using TP = typename std::remove_reference_t<decltype(DP)>::value_type;
          if constexpr (std::is_same<T, TP>::value)
            launch_overlap<T>(DG, DP, o.dst, o.src, o.fac, o.n, c->P, c->stream);
        });
      });
    }
}

void enqueue_movco(mge_ctx* c, int mgl) {  // movco.f90:21-47
  for (Block& b : c->lv[mgl - 1]) {
    cudaMemsetAsync(b.marker, 0, (size_t)b.N, c->stream);
    if ((int)c->lv.size() > mgl)
      for (Block& f : c->lv[mgl])
        if (f.parent == b.serial) enqueue_collc(c, b, f);
    enqueue_simple(c, b, 0);
    enqueue_simple(c, b, 1);
  }
  enqueue_overlap(c, mgl);
  for (Block& b : c->lv[mgl - 1]) enqueue_simple(c, b, 2);
}

void enqueue_movfin(mge_ctx* c, int mgl, int mlvl) {  // movfin.f90:20-39
  const bool fmg = (mgl - 1 == mlvl);
  for (Block& f : c->lv[mgl - 1]) {
    if (f.parent < 1) continue;
    Block& pb = c->lv[mgl - 2][f.parent - 1];
    enqueue_addw_embed(c, f, pb, fmg, false);
  }
  for (Block& f : c->lv[mgl - 1]) enqueue_simple(c, f, 0);
  for (Block& f : c->lv[mgl - 1]) {  // bc_embed
    if (f.parent < 1) continue;
    Block& pb = c->lv[mgl - 2][f.parent - 1];
    enqueue_addw_embed(c, f, pb, fmg, true);
  }
  enqueue_overlap(c, mgl);
  for (Block& f : c->lv[mgl - 1]) enqueue_simple(c, f, 2);
}

// solver.f90:127-234, one multigrid cycle at FMG level mlvl (enqueue only)
void enqueue_cycle(mge_ctx* c, int mlvl) {
  const mge_params& P = c->prm;
  std::vector<int> icyc(c->lv.size() + 2, 0);
  int mgl = mlvl;
  for (;;) {    // lopmg
    for (;;) {  // lopr
      icyc[mgl] += 1;
      bool lfir = (mgl != mlvl);
      for (Block& b : c->lv[mgl - 1]) {  // solver.f90:151-158
        enqueue_euler(c, b, mgl, mlvl, false, lfir, 0, mgl == mlvl, true);
        enqueue_overlap(c, mgl);
      }
      if (mlvl == 1) return;
      for (Block& b : c->lv[mgl - 1]) {  // solver.f90:197-201
        enqueue_euler(c, b, mgl, mlvl, true, false, 0, false);
        enqueue_overlap(c, mgl);
      }
      mgl = mgl - 1;
      enqueue_movco(c, mgl);
      if (mgl == 1) break;
    }
    bool lfir = true;
    for (;;) {  // lopp
      for (Block& b : c->lv[mgl - 1]) {  // solver.f90:215-222
        enqueue_euler(c, b, mgl, mlvl, false, lfir, 0, false, true);
        enqueue_overlap(c, mgl);
      }
      lfir = false;
      mgl = mgl + 1;
      enqueue_movfin(c, mgl, mlvl);
      if (mgl == mlvl) return;
      if (icyc[mgl] != P.mgtype) break;  // cycle lopmg
      icyc[mgl] = 0;
    }
  }
}

void build_phys(mge_ctx* c) {
  const mge_params& P = c->prm;
  PhysParams& Q = c->P;
  Q.gamma = P.gamma;
  Q.gm1 = P.gamma - 1.0;
  Q.gm = 1.0 / (P.gamma - 1.0);
  Q.vis2 = P.vis2;
  Q.vis4 = P.vis4;
  Q.cfl = P.cfl;
  Q.dimcfl = P.cfl > 1.0 ? P.cfl - 1.0 : 0.0;
  Q.rho0 = P.rho0;
  Q.p0 = P.p0;
  Q.c0 = P.c0;
  Q.u0[0] = P.u0;
  Q.u0[1] = P.v0;
  Q.u0[2] = P.w0;
  Q.e0 = P.rho0 * P.h0 - P.p0;
  Q.si_far = std::pow(P.rho0, P.gamma) / P.p0;
  Q.matrix = P.dissip == MGE_DISSIP_MATRIX;
  Q.eqn_ns = P.eqntype == MGE_EQN_NS;
  Q.smoo = P.smoo;
  Q.vt = P.vt;
  Q.distype = P.distype;
  Q.irs_kind = P.irs_variant;
  Q.unsteady = P.execmode == 1;
  Q.gamma14 = P.gamma == 1.4;
  Q.pow_dg = std::fma(P.gamma, 5.0, -7.0) / 5.0;    // exact 5*gamma - 7, then /5
  Q.pow_dm = Q.gm - 2.5;                            // exact: both near 2.5
  Q.dtstep = P.dtstep;
  Q.viscl = P.viscl;
  Q.gas_const = P.gas_const;
  Q.prlmean = P.prlmean;
  Q.kt = P.viscl * P.gamma * P.gas_const / ((P.gamma - 1.0) * P.prlmean);
  Q.cfac = P.distype == MGE_DIS_CENTRAL ? 4.0 : (P.distype == MGE_DIS_ROE2 ? 1.0 : 2.0);
  Q.epsentr = P.epsentr;
  const double u0n = std::sqrt(P.u0 * P.u0 + P.v0 * P.v0 + P.w0 * P.w0);
  const double ref[5] = {P.rho0, u0n, u0n, u0n, P.p0};
  for (int q = 0; q < 5; q++) Q.lim_e2[q] = 1e-6 * ref[q] * ref[q] / (P.limfac > 0.0 ? P.limfac : 1.0);
  Q.rgm1 = 1.0 / (P.gamma - 1.0);
  Q.rgm1f = 1.0f / ((float)P.gamma - 1.0f);
  Q.rgamma = 1.0 / P.gamma;
  Q.rgammaf = 1.0f / (float)P.gamma;
}

// psmoo.f90:136-166 pivots for a line of l-1 unknowns (rows 2..l)
void irs_pivots(double smoo, int lm, int l, std::vector<double>& e1, std::vector<double>& e1r, std::vector<double>& e2) {
  const double aa = 1.0 + 2.0 * smoo, bb = -smoo;
  e1.assign(l + 2, 1.0);
  e2.assign(l + 2, 0.0);
  e1r.assign(l + 2, 1.0);
  e1[2] = aa;
  e2[2] = bb / aa;
  for (int q = 3; q <= lm; q++) {
    e1[q] = aa - bb * e2[q - 1];
    e2[q] = bb / e1[q];
  }
  e1[l] = aa - bb * e2[lm];
  for (int q = 0; q <= l; q++) e1r[q] = 1.0 / e1[q];
}

int valloc(mge_ctx* c, void** p, size_t n, size_t esz) {
  uint8_t* q = nullptr;
  int rc = dalloc(c, &q, n * esz);
  if (rc) return rc;
  *p = q;
  cudaError_t e = cudaMemset(q, 0, std::max<size_t>(n * esz, 1));
  return e == cudaSuccess ? MGE_OK : cuda_fail(c, e, "cudaMemset");
}

template <typename T>
void fill_view(Block& b, DevBlock<T>& d, void* scratch) {
  const long long N = b.N;
  std::memset(&d, 0, sizeof(d));
  d.nx = b.nx; d.ny = b.ny; d.nz = b.nz;
  d.il = b.il; d.jl = b.jl; d.kl = b.kl; d.ie = b.ie; d.je = b.je; d.ke = b.ke; d.ib = b.ib; d.jb = b.jb; d.kb = b.kb;
  d.Pi = b.Pi; d.Pj = b.Pj; d.N = N;
  d.w = (T*)b.w; d.p = (T*)b.p; d.wn = (T*)b.wn; d.ws = (T*)b.ws; d.dw = (T*)b.dw; d.fw = (T*)b.fw;
  d.w1 = (T*)b.w1; d.w2 = (T*)b.w2;
  d.wr = (T*)b.wr; d.qf = (T*)b.qf; d.vdtim = (T*)b.vdtim; d.lam = (T*)b.lam; d.dtim = b.dtim;
  d.blank = b.blank; d.marker = b.marker; d.cutmap = b.cutmap;
  d.eps = (T*)b.eps;
  T* sc = (T*)scratch;
  d.H = sc;
  d.F = sc + N;
  d.fp = sc + 16 * N;
  d.efs = sc + 19 * N;
  d.dfs = sc + 34 * N;
  d.dlt = sc + 49 * N;
  d.vt = sc + 64 * N;
  d.vfs = sc + 68 * N;
  d.hx = b.h[0];
  d.hy = b.h[1];
  d.hz = b.h[2];
  for (int q = 0; q < 3; q++) {
    d.rh[q] = 1.0 / b.h[q];
    d.r4h[q] = 1.0 / (4.0 * b.h[q]);
    d.rhf[q] = 1.0f / (float)b.h[q];
    d.r4hf[q] = 1.0f / (4.0f * (float)b.h[q]);
  }
  for (int q = 0; q < 3; q++) {
    d.s[q] = b.s[q];
    d.sqrt_ds[q] = std::sqrt(b.s[q] * b.s[q]);
  }
  d.vol = b.vol;
  d.rvol = 1.0 / b.vol;
  d.rvolf = 1.0f / (float)b.vol;
  d.nmir = (int)b.recs.size();
  d.m0 = b.m0;
  d.rec_i = b.rec_i; d.rec_cloud = b.rec_cloud; d.rec_coef = b.rec_coef; d.rec_nvec = b.rec_nvec;
  d.rec_qb = b.rec_qb; d.rec_area = b.rec_area; d.rec_wsol = (T*)b.rec_wsol; d.rec_psol = (T*)b.rec_psol;
  d.rec_wall = (T*)b.rec_wall; d.tgt_off = b.tgt_off; d.tgt_ops = b.tgt_ops;
  for (int f = 0; f < 6; f++) {
    d.bctype[f] = b.bctype[f];
    for (int q = 0; q < 3; q++) d.fnv[f][q] = b.fnv[f][q];
  }
}

// Whether a record's wall face counts in the wall forces: blocks of one
// level may overlap, and a wall face inside the physical cells of a block of
// lower serial is that block's to count (each face once)
bool record_counted(const mge_ctx* c, const Block& b, const int* ccid) {
  for (const Block& o : c->lv[b.level - 1]) {
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

int commit_block(mge_ctx* c, Block& b, double* scratch) {
  const long long N = b.N;
  const size_t es = b.esz;
  int rc;
  if ((rc = valloc(c, &b.w, 5 * N, es)) || (rc = valloc(c, &b.p, N, es)) || (rc = valloc(c, &b.wn, 5 * N, es)) ||
      (rc = valloc(c, &b.ws, 5 * N, es)) || (rc = valloc(c, &b.dw, 5 * N, es)) || (rc = valloc(c, &b.fw, 5 * N, es)) ||
      (rc = valloc(c, &b.wr, 5 * N, es)) || (rc = valloc(c, &b.qf, 5 * N, es)) || (rc = valloc(c, &b.vdtim, N, es)) ||
      (rc = valloc(c, &b.lam, N, es)) || (rc = dalloc(c, &b.dtim, 1)) || (rc = dalloc(c, &b.blank, N)) ||
      (rc = dalloc(c, &b.marker, N)) || (rc = dalloc(c, &b.cutmap, N)))
    return rc;
  if (c->prm.irs_variant == 1 && (rc = valloc(c, &b.eps, 3 * N, es))) return rc;
  if (c->prm.execmode == 1 && ((rc = valloc(c, &b.w1, 5 * N, es)) || (rc = valloc(c, &b.w2, 5 * N, es)))) return rc;
  CK(cudaMemset(b.marker, 0, N));
  std::vector<uint8_t> bl(N);
  for (long long q = 0; q < N; q++) bl[q] = b.blank_h[q] != 0 ? 1 : 0;
  CK(cudaMemcpy(b.blank, bl.data(), N, cudaMemcpyHostToDevice));
  // cut records
  const int nm = (int)b.recs.size();
  b.m0 = nm;
  for (int m = 0; m < nm; m++)
    if (b.recs[m].npoint == 0) {
      b.m0 = m;
      break;
    }
  std::vector<int32_t> ri(8 * std::max(nm, 1), 0), rcl(24 * std::max(nm, 1), 0);
  std::vector<double> rcf(8 * std::max(nm, 1), 0.0), rnv(3 * std::max(nm, 1), 0.0), rqb(3 * std::max(nm, 1), 0.0),
      rar(std::max(nm, 1), 0.0), rps(3 * std::max(nm, 1), 0.0);
  for (int m = 0; m < nm; m++) {
    const HRec& t = b.recs[m];
    ri[8 * m + 0] = t.ccid[0];
    ri[8 * m + 1] = t.ccid[1];
    ri[8 * m + 2] = t.ccid[2];
    ri[8 * m + 3] = t.faceid;
    ri[8 * m + 4] = t.zz;
    ri[8 * m + 5] = t.npoint;
    ri[8 * m + 6] = record_counted(c, b, t.ccid) ? 1 : 0;
    for (int q = 0; q < MGE_MAX_CLOUD; q++) {
      rcf[8 * m + q] = t.coef[q];
      for (int e = 0; e < 3; e++) rcl[(8 * m + q) * 3 + e] = t.ijk[q][e];
    }
    for (int e = 0; e < 3; e++) {
      rnv[3 * m + e] = t.nvec[e];
      rqb[3 * m + e] = t.qb[e];
      rps[3 * m + e] = t.psurf[e];
    }
    rar[m] = t.area;
  }
  b.cut_beside_bcond = nm > 0;
  for (int m = 0; m < nm && m < b.m0; m++)
    for (int q = 0; q < b.recs[m].npoint; q++) {
      const int* ijk = b.recs[m].ijk[q];
      if (ijk[0] < 2 || ijk[0] > b.il || ijk[1] < 2 || ijk[1] > b.jl || ijk[2] < 2 || ijk[2] > b.kl)
        b.cut_beside_bcond = false;
    }
  const int nma = std::max(nm, 1);
  if ((rc = dalloc(c, &b.rec_i, 8 * nma)) || (rc = dalloc(c, &b.rec_cloud, 24 * nma)) ||
      (rc = dalloc(c, &b.rec_coef, 8 * nma)) || (rc = dalloc(c, &b.rec_nvec, 3 * nma)) ||
      (rc = dalloc(c, &b.rec_qb, 3 * nma)) || (rc = dalloc(c, &b.rec_area, nma)) ||
      (rc = dalloc(c, &b.rec_psurf, 3 * nma)) || (rc = dalloc(c, &b.rec_pnew, 3 * nma)) ||
      (rc = valloc(c, &b.rec_wsol, 5 * nma, es)) || (rc = valloc(c, &b.rec_psol, nma, es)) ||
      (rc = valloc(c, &b.rec_wall, 25 * nma, es)))
    return rc;
  CK(cudaMemcpy(b.rec_i, ri.data(), ri.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b.rec_cloud, rcl.data(), rcl.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b.rec_coef, rcf.data(), rcf.size() * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b.rec_nvec, rnv.data(), rnv.size() * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b.rec_qb, rqb.data(), rqb.size() * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b.rec_area, rar.data(), rar.size() * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b.rec_psurf, rps.data(), rps.size() * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b.rec_pnew, rps.data(), rps.size() * 8, cudaMemcpyHostToDevice));
  // cut targets: per physical cell, the (record, role) ops in record order
  std::vector<int32_t> cutmap(N, -1);
  std::map<long long, std::vector<int32_t>> tg;
  auto phys = [&](int i, int j, int k) { return i >= 2 && i <= b.il && j >= 2 && j <= b.jl && k >= 2 && k <= b.kl; };
  std::vector<long long> order;
  for (int m = 0; m < nm; m++) {
    const HRec& t = b.recs[m];
    int d = t.zz - 1;
    int e[3] = {0, 0, 0};
    e[d] = t.faceid >= 4 ? -1 : 1;  // neighbour away from the wall
    int i = t.ccid[0], j = t.ccid[1], k = t.ccid[2];
    long long c0 = (long long)i + (long long)b.Pi * ((long long)j + (long long)b.Pj * k);
    if (phys(i, j, k)) {
      if (!tg.count(c0)) order.push_back(c0);
      tg[c0].push_back(2 * m);
    }
    int ni = i + e[0], nj = j + e[1], nk = k + e[2];
    long long c1 = (long long)ni + (long long)b.Pi * ((long long)nj + (long long)b.Pj * nk);
    if (phys(ni, nj, nk)) {
      if (!tg.count(c1)) order.push_back(c1);
      tg[c1].push_back(2 * m + 1);
    }
  }
  std::vector<int32_t> off(1, 0), ops;
  for (size_t t = 0; t < order.size(); t++) {
    cutmap[order[t]] = (int32_t)t;
    for (int32_t op : tg[order[t]]) ops.push_back(op);
    off.push_back((int32_t)ops.size());
  }
  if ((rc = dalloc(c, &b.tgt_off, off.size())) || (rc = dalloc(c, &b.tgt_ops, std::max<size_t>(ops.size(), 1))))
    return rc;
  CK(cudaMemcpy(b.cutmap, cutmap.data(), N * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b.tgt_off, off.data(), off.size() * 4, cudaMemcpyHostToDevice));
  if (!ops.empty()) CK(cudaMemcpy(b.tgt_ops, ops.data(), ops.size() * 4, cudaMemcpyHostToDevice));
  // IRS tables
  const int lens[3] = {b.il, b.jl, b.kl}, lms[3] = {b.nx, b.ny, b.nz};
  size_t tot = 0;
  for (int d = 0; d < 3; d++) tot += 3 * (size_t)(lens[d] + 2);
  if ((rc = dalloc(c, &b.irs, tot))) return rc;
  std::vector<double> all;
  size_t offs[3][3];
  for (int d = 0; d < 3; d++) {
    std::vector<double> e1, e1r, e2;
    irs_pivots(c->prm.smoo > 0.0 ? c->prm.smoo : 0.0, lms[d], lens[d], e1, e1r, e2);
    offs[d][0] = all.size();
    all.insert(all.end(), e1.begin(), e1.end());
    offs[d][1] = all.size();
    all.insert(all.end(), e1r.begin(), e1r.end());
    offs[d][2] = all.size();
    all.insert(all.end(), e2.begin(), e2.end());
  }
  CK(cudaMemcpy(b.irs, all.data(), all.size() * 8, cudaMemcpyHostToDevice));
  // single-precision tables: the FP32 sweeps then need no conversion per cell
  std::vector<float> all32(all.size());
  for (size_t q = 0; q < all.size(); q++) all32[q] = (float)all[q];
  for (int d = 0; d < 3; d++)
    for (int q = 0; q < lens[d] + 2; q++) all32[offs[d][1] + q] = 1.0f / all32[offs[d][0] + q];
  if ((rc = dalloc(c, &b.irs32, all32.size()))) return rc;
  CK(cudaMemcpy(b.irs32, all32.data(), all32.size() * 4, cudaMemcpyHostToDevice));
  for (int d = 0; d < 3; d++) {
    b.tabs[d].e1 = b.irs + offs[d][0];
    b.tabs[d].e1r = b.irs + offs[d][1];
    b.tabs[d].e2 = b.irs + offs[d][2];
    b.tabs[d].e1f = b.irs32 + offs[d][0];
    b.tabs[d].e1rf = b.irs32 + offs[d][1];
    b.tabs[d].e2f = b.irs32 + offs[d][2];
  }
  b.npart = rtrms_partials((long long)b.nx * b.ny * b.nz);
  if ((rc = dalloc(c, &b.rt_partial, b.npart)) || (rc = dalloc(c, &b.rt_cur, 1)) || (rc = dalloc(c, &b.forces, 8)))
    return rc;
  CK(cudaMemset(b.rt_cur, 0, 8));
  // kernel view
  if (b.f32)
    fill_view(b, b.dev32, scratch);
  else
    fill_view(b, b.dev, scratch);
  return MGE_OK;
}

}  // namespace

// ====================================================================== C-ABI
namespace {
void drop_group_plans(const mge_ctx* c);  // the group plans that hold this case (below)
}

extern "C" {

int mge_abi_version(void) { return MGE_ABI_VERSION; }

const char* mge_build_info(void) {
  return "code_mge_gb300 libmge_gpu: sm_103a, FP64 multigrid RK cycle, CUDA " MGE_STR(__CUDACC_VER_MAJOR__);
}

void mge_params_default(mge_params* p, double gamma, double mach, double alpha, double beta) {
  std::memset(p, 0, sizeof(*p));
  p->mstage = 5;
  const double cs[5] = {0.25, 1.0 / 6.0, 0.375, 0.5, 1.0}, cd[5] = {1.0, 0.0, 0.56, 0.0, 0.44};
  for (int q = 0; q < 5; q++) {
    p->cstp[q] = cs[q];
    p->cdis[q] = cd[q];
  }
  p->cfl = 2.8;
  p->vt = 0;
  p->vis2 = 0.5;
  p->vis4 = 0.5 / 32.0;
  p->smoo = 0.6;
  p->mgtype = 1;
  p->gamma = gamma;
  p->rm = mach;
  p->alpha = alpha;
  p->beta = beta;
  p->rho0 = 1.0;  // input_param.f90:61-69
  p->p0 = 1.0 / (gamma * std::pow(mach, 2.0));
  p->c0 = std::sqrt(gamma * p->p0 / p->rho0);
  p->ei0 = p->p0 / ((gamma - 1.0) * p->rho0);
  p->u0 = mach * p->c0 * std::cos(beta) * std::cos(alpha);
  p->v0 = mach * p->c0 * std::cos(beta) * std::sin(alpha);
  p->w0 = mach * p->c0 * std::sin(beta);
  p->h0 = gamma * p->ei0 + 0.5 * (p->u0 * p->u0 + p->v0 * p->v0 + p->w0 * p->w0);
  p->viscl = p->rho0 * p->u0 / 500.0;
  p->prlmean = 0.72;
  p->gas_const = p->p0 / p->rho0;
  p->limfac = 5.0;
  p->epsentr = 0.05;
  p->wall_adiabatic = 1;
  p->nlevel = 1;
  p->mcyc[0] = 100;
  p->conv_drop = 1.0e6;
}

int mge_init(const mge_params* prm, int device, mge_ctx** out) {
  if (!prm || !out) return MGE_EBADCFG;
  *out = nullptr;
  if (prm->nlevel < 1 || prm->nlevel > MGE_MAX_LEVEL || prm->mstage < 1 || prm->mstage > MGE_MAX_STAGE)
    return MGE_EBADCFG;
  if (prm->distype != MGE_DIS_CENTRAL && prm->distype != MGE_DIS_ROE1 && prm->distype != MGE_DIS_ROE2)
    return MGE_EBADCFG;
  if (prm->eqntype != MGE_EQN_EULER && prm->eqntype != MGE_EQN_NS) return MGE_EBADCFG;
  if (prm->dissip != MGE_DISSIP_SCALAR && prm->dissip != MGE_DISSIP_MATRIX) return MGE_EBADCFG;
  if (prm->irs_variant != 0 && prm->irs_variant != 1) return MGE_EBADCFG;
  if (prm->execmode != 0 && (prm->execmode != 1 || !(prm->dtstep > 0.0))) return MGE_EBADCFG;
  mge_ctx* c = new mge_ctx();
  {
    static std::atomic<unsigned long long> next_uid{1};
    c->uid = next_uid++;
  }
  c->prm = *prm;
  c->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_err, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemset(c->d_err, 0, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMallocHost(&c->h_err, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMallocHost(&c->h_rt, 64 * sizeof(double));
  if (e != cudaSuccess) {
    delete c;
    return MGE_ECUDA;
  }
  c->lv.resize(prm->nlevel);
  build_phys(c);
  if (const char* e = getenv("MGE_COOP_MAX_CELLS")) {
    c->coop_max_cells = atoll(e);
    c->tune_path = false;  // an explicit threshold fixes the launch form
  }
  if (const char* e = getenv("MGE_AUTOTUNE")) c->autotune = atoi(e) != 0;
  if (const char* e = getenv("MGE_COOP_MAX_CTAS")) c->coop_max_ctas = atoi(e);
  if (const char* e = getenv("MGE_TUNE_PLAN")) c->plan = e;
  *out = c;
  return MGE_OK;
}

void mge_destroy(mge_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  drop_group_plans(c);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->ev_group) cudaEventDestroy(c->ev_group);
  for (cudaGraphExec_t g : c->graphs)
    if (g) cudaGraphExecDestroy(g);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->ev_done) cudaEventDestroy(c->ev_done);
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
  if (c->side) cudaStreamDestroy(c->side);
  for (void* q : c->allocs) cudaFree(q);
  if (c->scratch) cudaFree(c->scratch);
  if (c->d_err) cudaFree(c->d_err);
  if (c->h_err) cudaFreeHost(c->h_err);
  if (c->h_rt) cudaFreeHost(c->h_rt);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* mge_last_error(const mge_ctx* c) { return c ? c->err.c_str() : "null context"; }

int mge_add_block(mge_ctx* c, const mge_block_desc* d, int level, int serial) {
  if (!c || !d) return MGE_EBADCFG;
  if (c->committed) return fail(c, MGE_EBADCFG, "add_block after commit");
  if (level < 1 || level > (int)c->lv.size()) return fail(c, MGE_EBADCFG, "add_block: bad level");
  auto& L = c->lv[level - 1];
  if (serial != (int)L.size() + 1) return fail(c, MGE_EBADCFG, "add_block: serials must be added in order");
  if (d->nx < 2 || d->ny < 2 || d->nz < 2) return fail(c, MGE_EBADCFG, "add_block: need at least 2 cells per axis");
  if (d->si[1] != 0.0 || d->si[2] != 0.0 || d->sj[0] != 0.0 || d->sj[2] != 0.0 || d->sk[0] != 0.0 || d->sk[1] != 0.0)
    return fail(c, MGE_EBADCFG, "add_block: face vectors must be axis-aligned (uniform Cartesian block)");
  for (int f = 0; f < 6; f++) {
    int t = d->bctype[f];
    if (t != 0 && t != -20 && t != -50 && t != -60 && t != -80)
      return fail(c, MGE_EBADCFG, "add_block: unsupported bctype");
    if (t == -60 && f < 3 && d->bctype[f + 3] != -60)
      return fail(c, MGE_EBADCFG, "periodic boundary must appear in pairs (bcond.f90:26-31)");
  }
  if (level > 1) {
    if (d->parent < 1 || d->parent > (int)c->lv[level - 2].size())
      return fail(c, MGE_EBADCFG, "add_block: parent block must be added first");
    for (int q = 0; q < 3; q++)
      if (d->ratio[q] != 1 && d->ratio[q] != 2) return fail(c, MGE_EBADCFG, "add_block: ratio must be 1 or 2");
    if (d->nx % d->ratio[0] || d->ny % d->ratio[1] || d->nz % d->ratio[2])
      return fail(c, MGE_EBADCFG, "add_block: cells not divisible by the ratio");
  }
  L.emplace_back();
  Block& b = L.back();
  b.level = level;
  b.serial = serial;
  b.nx = d->nx; b.ny = d->ny; b.nz = d->nz;
  b.il = b.nx + 1; b.jl = b.ny + 1; b.kl = b.nz + 1;
  b.ie = b.il + 1; b.je = b.jl + 1; b.ke = b.kl + 1;
  b.ib = b.il + 2; b.jb = b.jl + 2; b.kb = b.kl + 2;
  b.Pi = b.ib + 1; b.Pj = b.jb + 1; b.Pk = b.kb + 1;
  b.N = (long long)b.Pi * b.Pj * b.Pk;
  for (int q = 0; q < 3; q++) {
    b.h[q] = d->h[q];
    b.origin[q] = d->origin[q];
    b.ratio[q] = d->ratio[q];
    b.offset[q] = d->offset[q];
  }
  b.s[0] = d->si[0];
  b.s[1] = d->sj[1];
  b.s[2] = d->sk[2];
  b.vol = d->cellvolume;
  for (int f = 0; f < 6; f++) {
    b.bctype[f] = d->bctype[f];
    for (int q = 0; q < 3; q++) b.fnv[f][q] = d->facenvec[f][q];
  }
  b.parent = d->parent;
  b.blank_h.assign(b.N, 1);
  if (d->blank)
    for (long long q = 0; q < b.N; q++) b.blank_h[q] = d->blank[q];
  b.recs.resize(d->nmir);
  for (int m = 0; m < d->nmir; m++) {
    HRec& t = b.recs[m];
    for (int q = 0; q < 3; q++) {
      t.ccid[q] = d->ccid[3 * m + q];
      t.scid[q] = d->scid[3 * m + q];
      t.nvec[q] = d->nvec[3 * m + q];
      t.qb[q] = d->qb ? d->qb[3 * m + q] : 0.0;
      t.psurf[q] = d->psurf ? d->psurf[3 * m + q] : 0.0;
    }
    t.faceid = d->faceid[m];
    t.zz = d->zz[m];
    t.npoint = d->npoint[m];
    if (t.npoint < 0 || t.npoint > MGE_MAX_CLOUD) return fail(c, MGE_EBADCFG, "add_block: bad cloud size");
    if (t.zz < 1 || t.zz > 3 || t.faceid < 1 || t.faceid > 6 || (t.faceid - 1) % 3 != t.zz - 1)
      return fail(c, MGE_EBADCFG, "add_block: faceid/zz mismatch");
    int lim[3] = {b.ib, b.jb, b.kb}, phys_lo = 2, phys_hi[3] = {b.il, b.jl, b.kl};
    for (int q = 0; q < 3; q++)
      if (t.ccid[q] < phys_lo || t.ccid[q] > phys_hi[q]) return fail(c, MGE_EBADCFG, "add_block: cut cell not physical");
    // the dissipation stencils reach two cells beyond the cut cell along the record axis
    int ax = t.zz - 1;
    if (t.ccid[ax] - 2 < 0 || t.ccid[ax] + 2 > lim[ax]) return fail(c, MGE_EBADCFG, "add_block: record too close to edge");
    for (int q = 0; q < MGE_MAX_CLOUD; q++) {
      t.coef[q] = d->coef[MGE_MAX_CLOUD * m + q];
      for (int e = 0; e < 3; e++) {
        t.ijk[q][e] = d->ijkdex[(MGE_MAX_CLOUD * m + q) * 3 + e];
        if (q < t.npoint && (t.ijk[q][e] < 0 || t.ijk[q][e] > lim[e]))
          return fail(c, MGE_EBADCFG, "add_block: cloud cell outside the block");
      }
    }
    double fa = 1.0;
    for (int e = 0; e < 3; e++)
      if (e != ax) fa *= d->h[e];
    t.area = d->area ? d->area[m] : fa;
  }
  c->order.emplace_back(level, serial);
  return MGE_OK;
}

// Stencil of ghost cell (i,j,k) of block g on block p of the same level, the
// construction of the prolongation (cell centre, containing cell, base of the
// 2x2x2 stencil clamped to p's physical cells); false outside p's physical cells
static bool overlap_stencil(const Block& g, const Block& p, int i, int j, int k, int* sh, double* fac) {
  const int ic[3] = {i, j, k}, lc[3] = {p.il, p.jl, p.kl}, nc[3] = {p.nx, p.ny, p.nz};
  double xi[3];
  for (int d = 0; d < 3; d++) {
    const double x = g.origin[d] + ((double)ic[d] - 1.5) * g.h[d];
    const double u = (x - p.origin[d]) / p.h[d];
    if (u < 0.0 || u >= (double)nc[d]) return false;
    int s = (int)std::floor(u + 1.5);
    if (s < 2) s = 2;
    if (s > lc[d] - 1) s = lc[d] - 1;
    sh[d] = s;
    xi[d] = u + 1.5 - (double)s;
  }
  const double x = xi[0], y = xi[1], z = xi[2];
  fac[0] = (1.0 - x) * (1.0 - y) * (1.0 - z);
  fac[1] = x * (1.0 - y) * (1.0 - z);
  fac[2] = (1.0 - x) * y * (1.0 - z);
  fac[3] = x * y * (1.0 - z);
  fac[4] = (1.0 - x) * (1.0 - y) * z;
  fac[5] = x * (1.0 - y) * z;
  fac[6] = (1.0 - x) * y * z;
  fac[7] = x * y * z;
  return true;
}

// the overlap lists of every block (levels with one block have none)
static int build_overlaps(mge_ctx* c) {
  for (auto& L : c->lv) {
    if (L.size() < 2) continue;
    for (Block& g : L)
      for (Block& p : L) {
        if (&g == &p) continue;
        std::vector<long long> dst, src;
        std::vector<double> fac;
        for (int i = 0; i <= g.ib; i++)
          for (int j = 0; j <= g.jb; j++)
            for (int k = 0; k <= g.kb; k++) {
              if (i >= 2 && i <= g.il && j >= 2 && j <= g.jl && k >= 2 && k <= g.kl) continue;
              int sh[3];
              double f[8];
              if (!overlap_stencil(g, p, i, j, k, sh, f)) continue;
              dst.push_back((long long)i + (long long)g.Pi * (j + (long long)g.Pj * k));
              src.push_back((long long)sh[0] + (long long)p.Pi * (sh[1] + (long long)p.Pj * sh[2]));
              fac.insert(fac.end(), f, f + 8);
            }
        if (dst.empty()) continue;
        Block::Overlap o;
        o.partner = p.serial;
        o.n = (long long)dst.size();
        int rc;
        if ((rc = dalloc(c, &o.dst, dst.size())) || (rc = dalloc(c, &o.src, src.size())) ||
            (rc = dalloc(c, &o.fac, fac.size())))
          return rc;
        CK(cudaMemcpy(o.dst, dst.data(), dst.size() * sizeof(long long), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(o.src, src.data(), src.size() * sizeof(long long), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(o.fac, fac.data(), fac.size() * sizeof(double), cudaMemcpyHostToDevice));
        g.ovl.push_back(o);
      }
  }
  return MGE_OK;
}

// The contracted FP64 residual applies to the finest level of the mixed and
// refined forms, for the steady JST central scheme (scalar dissipation) of
// the Euler equations; MGE_FAST_RESIDUAL=0 turns it off.
static bool fast_residual(const mge_ctx* c, bool finest, int precision) {
  const char* e = getenv("MGE_FAST_RESIDUAL");
  if (e && e[0] == '0') return false;
  const mge_params& P = c->prm;
  return finest && precision != MGE_PREC_FP64 && P.distype == MGE_DIS_CENTRAL && P.eqntype == MGE_EQN_EULER &&
         P.dissip == MGE_DISSIP_SCALAR && P.execmode == 0;
}

int mge_commit(mge_ctx* c) {
  if (!c) return MGE_EBADCFG;
  if (c->committed) return MGE_OK;
  CK(cudaSetDevice(c->device));
  long long maxN = 0;
  for (auto& L : c->lv) {
    if (L.empty()) return fail(c, MGE_EBADCFG, "commit: a level has no block");
    for (Block& b : L) maxN = std::max(maxN, b.N);
  }
  init_kernel_attributes();
  // scratch: H(1) F(15) fp(3) efs(15) dfs(15) dlt(15) = 64 fields of the
  // largest block, + vt(4) vfs(15) for Navier-Stokes
  const size_t nsc = c->prm.eqntype == MGE_EQN_NS ? 83 : 64;
  int rc = dalloc(c, &c->scratch, nsc * maxN);
  if (rc) return rc;
  c->allocs.pop_back();  // freed separately
  const bool mixed = c->prm.precision == MGE_PREC_MIXED;
  for (size_t l = 0; l < c->lv.size(); l++)
    for (Block& b : c->lv[l]) {
      // mixed: coarse levels in FP32; the finest keeps FP64 state and residual,
      // with its time step and residual smoothing in FP32 arithmetic
      b.f32 = mixed && (l + 1 < c->lv.size());
      b.aux32 = mixed && !b.f32;
      b.fast = fast_residual(c, l + 1 == c->lv.size(), c->prm.precision);
      b.esz = b.f32 ? 4 : 8;
      b.use_coop = (long long)b.nx * b.ny * b.nz <= c->coop_max_cells;
      if ((rc = commit_block(c, b, c->scratch))) return rc;
    }
  if ((rc = build_overlaps(c))) return rc;
  // the set-up copies ran on the legacy stream; order them before the context stream
  CK(cudaDeviceSynchronize());
  c->committed = true;
  return MGE_OK;
}

static void free_stream_start(mge_ctx* c, Block& b) {  // init_flow.f90:46-96
  enqueue_simple(c, b, 3);
  enqueue_simple(c, b, 0);
  enqueue_simple(c, b, 4);
  enqueue_simple(c, b, 2);
  if (b.w1) {  // init_flow.f90:79-86: the previous time steps start equal to w
    cudaMemcpyAsync(b.w1, b.w, 5 * b.N * b.esz, cudaMemcpyDeviceToDevice, c->stream);
    cudaMemcpyAsync(b.w2, b.w, 5 * b.N * b.esz, cudaMemcpyDeviceToDevice, c->stream);
  }
}

// Autotuner: per block, time the two line-sweep variants of each direction
// and the two launch forms of one timestep + euler update (one cooperative
// launch, or one launch per phase) on the free-stream state, keep the faster,
// and cache the choice by block shape and precision for later contexts.
struct TuneKey {
  int nx, ny, nz, f32, aux32, rec, scheme;  // scheme: smoothing variant, equations, flux
  bool operator<(const TuneKey& o) const {
    return std::tie(nx, ny, nz, f32, aux32, rec, scheme) < std::tie(o.nx, o.ny, o.nz, o.f32, o.aux32, o.rec, o.scheme);
  }
};
struct TuneVal {
  bool coop;
  int irs[3];
};
static std::map<TuneKey, TuneVal> g_tune;
static std::mutex g_tune_mu;

static int autotune_block(mge_ctx* c, Block& b, bool tune_path) {
  const mge_params& prm = c->prm;
  TuneKey key{b.nx, b.ny, b.nz, (int)b.f32, (int)b.aux32, b.recs.empty() ? 0 : 1,
              100 * prm.irs_variant + 10 * prm.eqntype + prm.distype};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      if (tune_path) b.use_coop = it->second.coop;
      for (int d = 0; d < 3; d++) b.irs_var[d] = it->second.irs[d];
      return MGE_OK;
    }
  }
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  auto time_it = [&](auto&& fn, int reps) -> float {
    fn();
    cudaEventRecord(e0, c->stream);
    for (int r = 0; r < reps; r++) fn();
    cudaEventRecord(e1, c->stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    return ms;
  };
  if (c->prm.smoo > 0.0 && c->prm.irs_variant == 0) {  // the psmoo variant has one form
    for (int d = 0; d < 3; d++) {
      float best = 1e30f;
      int bv = 0;
      // variant 2, the warp-scan i sweep, exists for the FP32 sweeps (the
      // mixed form's finest level and its FP32 levels)
      const int nvar = (d == 0 && (b.aux32 || b.f32)) ? 3 : 2;
      for (int v = 0; v < nvar; v++) {
        int var[3] = {0, 0, 0};
        var[d] = v;
        float t = time_it([&] {
          with_dev(b, [&](auto& D) {
            using T = typename std::remove_reference_t<decltype(D)>::value_type;
            launch_irs_part<T>(d, D, c->P, b.tabs, c->stream, b.aux32, var);
          });
        }, 3);
        if (t < best) {
          best = t;
          bv = v;
        }
      }
      b.irs_var[d] = bv;
    }
    free_stream_start(c, b);  // the timed sweeps ended in an update: restore the start state
  }
  if (tune_path) {
    float tc = 1e30f, tp = 1e30f;
    b.use_coop = true;
    tc = time_it([&] { enqueue_euler(c, b, b.level, b.level, false, false, 0, false, true); }, 2);
    cudaError_t e = cudaGetLastError();
    b.use_coop = false;
    tp = time_it([&] { enqueue_euler(c, b, b.level, b.level, false, false, 0, false, true); }, 2);
    b.use_coop = (e == cudaSuccess) && tc < tp;
    free_stream_start(c, b);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CK(cudaGetLastError());
  int rc = check_err(c);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = TuneVal{b.use_coop, {b.irs_var[0], b.irs_var[1], b.irs_var[2]}};
  return MGE_OK;
}

int mge_init_flow(mge_ctx* c) {  // init_flow.f90:46-96
  if (!c || !c->committed) return MGE_EBADCFG;
  CK(cudaSetDevice(c->device));
  for (auto& L : c->lv)
    for (Block& b : L) free_stream_start(c, b);
  c->itime = 0;
  CK(cudaGetLastError());
  int rc = check_err(c);
  if (rc) return rc;
  // a fixed plan "level:CIJK,..." (C = 1 cooperative euler, I/J/K = line-sweep
  // form per direction: 0 global lines, 1 shared-memory tiles, 2 the mixed
  // form's warp-scan i sweep) replaces tuning for the levels it names, so that a
  // run can repeat the launch forms another run chose
  std::vector<bool> fixed(c->lv.size(), false);
  for (size_t pos = 0; pos < c->plan.size();) {
    size_t end = c->plan.find(',', pos);
    if (end == std::string::npos) end = c->plan.size();
    const std::string item = c->plan.substr(pos, end - pos);
    pos = end + 1;
    const size_t colon = item.find(':');
    if (colon == std::string::npos || item.size() != colon + 5) return fail(c, MGE_EBADCFG, "MGE_TUNE_PLAN: bad item " + item);
    const int lvl = atoi(item.substr(0, colon).c_str());
    if (lvl < 1 || lvl > (int)c->lv.size()) return fail(c, MGE_EBADCFG, "MGE_TUNE_PLAN: bad level " + item);
    for (Block& b : c->lv[lvl - 1]) {
      b.use_coop = item[colon + 1] == '1';
      for (int d = 0; d < 3; d++) {
        const char f = item[colon + 2 + d];
        b.irs_var[d] = (f == '1' || f == '2') ? f - '0' : 0;
      }
    }
    fixed[lvl - 1] = true;
  }
  if (!c->autotune) return MGE_OK;
  for (size_t l = 0; l < c->lv.size(); l++)
    for (Block& b : c->lv[l]) {
      if (fixed[l]) continue;
      const bool tune_path = c->tune_path && (long long)b.nx * b.ny * b.nz <= 2000000;
      if ((rc = autotune_block(c, b, tune_path))) return rc;
    }
  return MGE_OK;
}

// free one allocation made by dalloc
static void dfree(mge_ctx* c, void* p, size_t bytes) {
  if (!p) return;
  auto it = std::find(c->allocs.begin(), c->allocs.end(), p);
  if (it != c->allocs.end()) c->allocs.erase(it);
  cudaFree(p);
  c->bytes -= std::min(c->bytes, bytes);
}

// Switch a context between the plain FP64 and the mixed form in place: coarse
// blocks change their storage (state converted, scratch fields re-zeroed),
// the finest block toggles its FP32 time step and smoothing.
int mge_set_precision(mge_ctx* c, int precision) {
  if (!c || !c->committed ||
      (precision != MGE_PREC_FP64 && precision != MGE_PREC_MIXED && precision != MGE_PREC_REFINED))
    return MGE_EBADCFG;
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  const bool mixed = precision == MGE_PREC_MIXED;
  for (size_t l = 0; l < c->lv.size(); l++)
    for (Block& b : c->lv[l]) {
      const bool finest = l + 1 == c->lv.size();
      const bool f32 = mixed && !finest;
      b.aux32 = precision != MGE_PREC_FP64 && finest;
      b.fast = fast_residual(c, finest, precision);
      if (f32 == b.f32) continue;
      const size_t oes = b.esz, nes = f32 ? 4 : 8;
      const long long N = b.N;
      const int nma = std::max((int)b.recs.size(), 1);
      struct F { void** p; long long n; bool keep; };
      F fields[] = {{&b.w, 5 * N, true},  {&b.p, N, true},        {&b.ws, 5 * N, true},   {&b.wn, 5 * N, false},
                    {&b.dw, 5 * N, false}, {&b.fw, 5 * N, false}, {&b.wr, 5 * N, false}, {&b.qf, 5 * N, false},
                    {&b.vdtim, N, false}, {&b.lam, N, false},     {&b.rec_wsol, 5LL * nma, true},
                    {&b.rec_psol, nma, true}, {&b.rec_wall, 25LL * nma, false}, {&b.eps, 3 * N, false},
                    {&b.w1, 5 * N, true},     {&b.w2, 5 * N, true}};
      for (F& f : fields) {
        if (!*f.p) continue;  // not allocated for this context
        void* np = nullptr;
        int rc = valloc(c, &np, (size_t)f.n, nes);
        if (rc) return rc;
        if (f.keep) launch_convert(*f.p, oes == 4, np, nes == 4, f.n, c->stream);
        CK(cudaStreamSynchronize(c->stream));
        dfree(c, *f.p, (size_t)f.n * oes);
        *f.p = np;
      }
      b.f32 = f32;
      b.esz = nes;
      if (b.f32)
        fill_view(b, b.dev32, c->scratch);
      else
        fill_view(b, b.dev, c->scratch);
    }
  for (cudaGraphExec_t& g : c->graphs)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  c->prm.precision = precision;
  c->gen++;  // group plans holding this case's old fields are stale
  CK(cudaGetLastError());
  return check_err(c);
}

int mge_tuned(mge_ctx* c, int level, int serial, int* coop, int* irs3) {
  Block* b = getb(c, level, serial);
  if (!b) return MGE_ENOTFOUND;
  if (coop) *coop = b->use_coop ? 1 : 0;
  if (irs3)
    for (int d = 0; d < 3; d++) irs3[d] = b->irs_var[d];
  return MGE_OK;
}

int mge_upload_state(mge_ctx* c, int level, int serial, const double* w) {
  Block* b = getb(c, level, serial);
  if (!b || !c->committed) return MGE_ENOTFOUND;
  CK(cudaSetDevice(c->device));
  if (b->f32) {
    std::vector<float> t(5 * b->N);
    for (long long q = 0; q < 5 * b->N; q++) t[q] = (float)w[q];
    CK(cudaMemcpyAsync(b->w, t.data(), t.size() * 4, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  } else {
    CK(cudaMemcpyAsync(b->w, w, 5 * b->N * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  }
  // what init_flow.f90:46-66 does after read_solut: depvars, bc_cutcell (the
  // records' solid state from the new cells), bcond
  enqueue_simple(c, *b, 0);
  enqueue_simple(c, *b, 4);
  enqueue_simple(c, *b, 2);
  return check_err(c);
}

// copy len values of a state field (double, or float when the block is FP32) to host doubles
static int copy_out(mge_ctx* c, const Block& b, const void* src, size_t len, bool typed, double* out) {
  if (!len) return MGE_OK;
  if (typed && b.f32) {
    std::vector<float> t(len);
    CK(cudaMemcpy(t.data(), src, len * 4, cudaMemcpyDeviceToHost));
    for (size_t q = 0; q < len; q++) out[q] = (double)t[q];
  } else {
    CK(cudaMemcpy(out, src, len * sizeof(double), cudaMemcpyDeviceToHost));
  }
  return MGE_OK;
}

int mge_download_state(mge_ctx* c, int level, int serial, double* w, double* p) {
  Block* b = getb(c, level, serial);
  if (!b || !c->committed) return MGE_ENOTFOUND;
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  int rc = MGE_OK;
  if (w && (rc = copy_out(c, *b, b->w, 5 * b->N, true, w))) return rc;
  if (p && (rc = copy_out(c, *b, b->p, b->N, true, p))) return rc;
  return MGE_OK;
}

int mge_download_field(mge_ctx* c, int level, int serial, const char* name, double* out, size_t count) {
  Block* b = getb(c, level, serial);
  if (!b || !c->committed || !name) return MGE_ENOTFOUND;
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  std::string n(name);
  const long long N = b->N;
  const void* src = nullptr;
  size_t len = 0;
  bool typed = true;
  if (n == "w") { src = b->w; len = 5 * N; }
  else if (n == "p") { src = b->p; len = N; }
  else if (n == "dw") { src = b->dw; len = 5 * N; }
  else if (n == "fw") { src = b->fw; len = 5 * N; }
  else if (n == "wn") { src = b->wn; len = 5 * N; }
  else if (n == "ws") { src = b->ws; len = 5 * N; }
  else if (n == "wr") { src = b->wr; len = 5 * N; }
  else if (n == "qf") { src = b->qf; len = 5 * N; }
  else if (n == "vdtim") { src = b->vdtim; len = N; }
  else if (n == "lam") { src = b->lam; len = N; }
  else if (n == "eps" && b->eps) { src = b->eps; len = 3 * N; }
  else if (n == "w1" && b->w1) { src = b->w1; len = 5 * N; }
  else if (n == "w2" && b->w2) { src = b->w2; len = 5 * N; }
  else if (n == "wsol") { src = b->rec_wsol; len = 5 * b->recs.size(); }
  else if (n == "psol") { src = b->rec_psol; len = b->recs.size(); }
  else if (n == "dtim") { src = b->dtim; len = 1; typed = false; }
  if (src) {
    if (count < len) return fail(c, MGE_EBADCFG, "download_field: buffer too small");
    return copy_out(c, *b, src, len, typed, out);
  }
  if (n == "blank" || n == "marker") {
    if (count < (size_t)N) return fail(c, MGE_EBADCFG, "download_field: buffer too small");
    std::vector<uint8_t> t(N);
    CK(cudaMemcpy(t.data(), n == "blank" ? b->blank : b->marker, N, cudaMemcpyDeviceToHost));
    for (long long q = 0; q < N; q++) out[q] = (double)t[q];
    return MGE_OK;
  }
  return fail(c, MGE_EBADCFG, "download_field: unknown field " + n);
}

int mge_timestep(mge_ctx* c, int level, int serial) {
  Block* b = getb(c, level, serial);
  if (!b || !c->committed) return MGE_ENOTFOUND;
  CK(cudaSetDevice(c->device));
  enqueue_timestep(c, *b);
  CK(cudaGetLastError());
  return check_err(c);
}

static int euler_common(mge_ctx* c, int level, int serial, int itime, int ncyc, int mgl, int mlvl, int lres,
                        int lfir, int nstage) {
  Block* b = getb(c, level, serial);
  if (!b || !c->committed) return MGE_ENOTFOUND;
  CK(cudaSetDevice(c->device));
  const bool full = !lres && (nstage <= 0 || nstage >= c->prm.mstage);
  enqueue_euler(c, *b, mgl, mlvl, lres != 0, lfir != 0, nstage, full, false, itime < 0 ? 0 : itime);
  CK(cudaGetLastError());
  int rc = check_err(c);
  if (rc) return rc;
  if (full && ncyc >= 0) {
    double v = 0.0;
    CK(cudaMemcpy(&v, b->rt_cur, sizeof(double), cudaMemcpyDeviceToHost));
    if ((int)b->rtrms.size() <= ncyc) b->rtrms.resize(ncyc + 1, 0.0);
    b->rtrms[ncyc] = v;
  }
  return MGE_OK;
}

int mge_euler(mge_ctx* c, int level, int serial, int itime, int ncyc, int mgl, int mlvl, int lres, int lfir) {
  return euler_common(c, level, serial, itime, ncyc, mgl, mlvl, lres, lfir, 0);
}

int mge_euler_partial(mge_ctx* c, int level, int serial, int itime, int ncyc, int mgl, int mlvl, int lres, int lfir,
                      int nstage) {
  return euler_common(c, level, serial, itime, ncyc, mgl, mlvl, lres, lfir, nstage);
}

int mge_movco(mge_ctx* c, int mgl) {
  if (!c || !c->committed || mgl < 1 || mgl > (int)c->lv.size()) return MGE_ENOTFOUND;
  CK(cudaSetDevice(c->device));
  enqueue_movco(c, mgl);
  CK(cudaGetLastError());
  return check_err(c);
}

int mge_movfin(mge_ctx* c, int mgl, int mlvl) {
  if (!c || !c->committed || mgl < 2 || mgl > (int)c->lv.size()) return MGE_ENOTFOUND;
  CK(cudaSetDevice(c->device));
  enqueue_movfin(c, mgl, mlvl);
  CK(cudaGetLastError());
  return check_err(c);
}

int mge_bc_overlap(mge_ctx* c, int mgl) {
  if (!c || !c->committed || mgl < 1 || mgl > (int)c->lv.size()) return MGE_ENOTFOUND;
  CK(cudaSetDevice(c->device));
  enqueue_overlap(c, mgl);
  CK(cudaGetLastError());
  return check_err(c);
}

int mge_get_rtrms(mge_ctx* c, int level, int serial, int ncyc, double* out) {
  Block* b = getb(c, level, serial);
  if (!b || !out) return MGE_ENOTFOUND;
  *out = (ncyc >= 0 && ncyc < (int)b->rtrms.size()) ? b->rtrms[ncyc] : 0.0;
  return MGE_OK;
}

// upload_solut.f90:203-237 on the device: the output variables of one block's
// physical cells, computed in the stage scratch and copied to the caller
int mge_upload_solut(mge_ctx* c, int level, int serial, double p_tot, double* solut, size_t count, int* nval_out) {
  Block* b = getb(c, level, serial);
  if (!b || !c->committed) return MGE_ENOTFOUND;
  const int ns = c->prm.eqntype == MGE_EQN_NS ? 1 : 0;
  const int nval = ns ? 11 : 7;
  if (nval_out) *nval_out = nval;
  const size_t ncell = (size_t)b->nx * b->ny * b->nz;
  if (!solut || count < nval * ncell) return fail(c, MGE_EBADCFG, "upload_solut: buffer too small");
  CK(cudaSetDevice(c->device));
  // the scratch holds at least 64 fields of the largest block: room for 11
  with_dev(*b, [&](auto& D) {
    using T = typename std::remove_reference_t<decltype(D)>::value_type;
    launch_solut<T>(D, c->P, c->prm.rm, p_tot, ns, c->scratch, c->stream);
  });
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(solut, c->scratch, nval * ncell * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return check_err(c);
}

// write_solut / read_solut (wsolut.f90:49-92, rsolut.f90:1-41): every block
// of the context, in mge_add_block order, as the reference's restart text.
// codes[q] is the block code of the q-th block added (ncodes = 0: 1, 2, ...).
int mge_write_restart(mge_ctx* c, const char* path, const int* codes, int ncodes) {
  if (!c || !c->committed || !path) return MGE_EBADCFG;
  if (ncodes != 0 && (ncodes != (int)c->order.size() || !codes)) return fail(c, MGE_EBADCFG, "write_restart: codes");
  FILE* f = std::fopen(path, "w");
  if (!f) return fail(c, MGE_EBADCFG, std::string("write_restart: cannot open ") + path);
  int rc = MGE_OK;
  std::vector<double> w, p;
  std::vector<char> text;
  for (size_t q = 0; q < c->order.size() && !rc; q++) {
    Block* b = getb(c, c->order[q].first, c->order[q].second);
    w.resize(5 * b->N);
    p.resize(b->N);
    rc = mge_download_state(c, c->order[q].first, c->order[q].second, w.data(), p.data());
    if (rc) break;
    const int code = ncodes ? codes[q] : (int)q + 1;
    const long long need = mge_restart_format(code, b->ib, b->jb, b->kb, w.data(), nullptr, 0);
    text.resize((size_t)need + 1);
    mge_restart_format(code, b->ib, b->jb, b->kb, w.data(), text.data(), need + 1);
    if (std::fwrite(text.data(), 1, (size_t)need, f) != (size_t)need) rc = fail(c, MGE_EBADCFG, "write_restart: write");
  }
  std::fclose(f);
  return rc;
}

int mge_read_restart(mge_ctx* c, const char* path, const int* codes, int ncodes) {
  if (!c || !c->committed || !path) return MGE_EBADCFG;
  if (ncodes != 0 && (ncodes != (int)c->order.size() || !codes)) return fail(c, MGE_EBADCFG, "read_restart: codes");
  FILE* f = std::fopen(path, "r");
  if (!f) return fail(c, MGE_EBADCFG, std::string("read_restart: cannot open ") + path);
  std::string text;
  char chunk[1 << 16];
  size_t got;
  while ((got = std::fread(chunk, 1, sizeof chunk, f)) > 0) text.append(chunk, got);
  std::fclose(f);
  long long pos = 0;
  std::vector<double> w;
  for (size_t q = 0; q < c->order.size(); q++) {
    Block* b = getb(c, c->order[q].first, c->order[q].second);
    w.resize(5 * b->N);
    const int code = ncodes ? codes[q] : (int)q + 1;
    const long long used =
        mge_restart_parse(text.data() + pos, (long long)text.size() - pos, code, b->ib, b->jb, b->kb, w.data());
    if (used < 0) return fail(c, MGE_EBADCFG, "read_restart: inconsistent file dof & grid dimension (rsolut.f90:27-32)");
    pos += used;
    int rc = mge_upload_state(c, c->order[q].first, c->order[q].second, w.data());
    if (rc) return rc;
  }
  return MGE_OK;
}

// solver.f90:263-276,286: the end of a physical time step of the unsteady
// mode: w2 = w1, w1 = w on every block, and the step counter advances
int mge_time_advance(mge_ctx* c, int* itime_out) {
  if (!c || !c->committed) return MGE_EBADCFG;
  if (c->prm.execmode != 1) return fail(c, MGE_EBADCFG, "time_advance: execmode is not 1");
  CK(cudaSetDevice(c->device));
  for (auto& L : c->lv)
    for (Block& b : L) {
      CK(cudaMemcpyAsync(b.w2, b.w1, 5 * b.N * b.esz, cudaMemcpyDeviceToDevice, c->stream));
      CK(cudaMemcpyAsync(b.w1, b.w, 5 * b.N * b.esz, cudaMemcpyDeviceToDevice, c->stream));
    }
  CK(cudaStreamSynchronize(c->stream));
  c->itime += 1;
  if (itime_out) *itime_out = c->itime;
  return MGE_OK;
}

int mge_move_surface(mge_ctx* c, int level, int serial, const double* disp, const double* norv, const double* vel,
                     double vel_fs) {
  Block* b = getb(c, level, serial);
  if (!b || !c->committed) return MGE_ENOTFOUND;
  if (c->group_pending) return fail(c, MGE_EBADCFG, "move_surface: a group cycle is in flight");
  if (!(vel_fs > 0.0)) return fail(c, MGE_EBADCFG, "move_surface: vel_fs must be positive");
  const long long nm = (long long)b->recs.size();
  if (!nm) return MGE_OK;
  if (!disp || !norv || !vel) return fail(c, MGE_EBADCFG, "move_surface: null record array");
  CK(cudaSetDevice(c->device));
  // queued behind the context's earlier work, so a cycle in flight sees the
  // old surface and the next one the new
  CK(cudaMemcpyAsync(b->rec_nvec, norv, 3 * nm * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(b->rec_pnew, disp, 3 * nm * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(b->rec_qb, vel, 3 * nm * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  launch_movsurf(nm, b->rec_psurf, b->rec_pnew, b->rec_qb, vel_fs, c->stream);
  CK(cudaGetLastError());
  return check_err(c);
}

int mge_get_surface(mge_ctx* c, int level, int serial, double* pnew) {
  Block* b = getb(c, level, serial);
  if (!b || !c->committed || !pnew) return MGE_ENOTFOUND;
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaMemcpy(pnew, b->rec_pnew, 3 * b->recs.size() * sizeof(double), cudaMemcpyDeviceToHost));
  return check_err(c);
}

int mge_forces_compute(mge_ctx* c, int level, const mge_solve_opts* o, mge_forces* out) {
  if (!c || !c->committed || level < 1 || level > (int)c->lv.size() || !out) return MGE_ENOTFOUND;
  CK(cudaSetDevice(c->device));
  double F[3] = {0, 0, 0}, M[3] = {0, 0, 0};
  const double ctr[3] = {o ? o->moment_center[0] : 0.0, o ? o->moment_center[1] : 0.0, o ? o->moment_center[2] : 0.0};
  for (Block& b : c->lv[level - 1]) {
    if (b.recs.empty()) continue;
    with_dev(b, [&](auto& D) {
      using T = typename std::remove_reference_t<decltype(D)>::value_type;
      launch_forces<T>(D, b.origin, b.h, ctr, c->prm.eqntype == MGE_EQN_NS ? c->prm.viscl : 0.0, b.forces,
                       c->stream);
    });
    double h6[8];
    CK(cudaMemcpyAsync(h6, b.forces, 6 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int d = 0; d < 3; d++) {
      F[d] += h6[d];
      M[d] += h6[3 + d];
    }
  }
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

static int launch_cycle_graph(mge_ctx* c, int mlvl_in) {
  // one graph per FMG level and, in the unsteady mode, per form of the
  // transient source (none, first step, BDF2): the stage arguments are baked in
  const int tclass = c->prm.execmode == 1 ? std::min(c->itime, 2) : 0;
  const int mlvl = mlvl_in + tclass * ((int)c->lv.size() + 1);
  if ((int)c->graphs.size() < 3 * ((int)c->lv.size() + 1)) c->graphs.resize(3 * (c->lv.size() + 1), nullptr);
  if (!c->graphs[mlvl]) {
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    enqueue_cycle(c, mlvl_in);
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&c->graphs[mlvl], g, 0);
    size_t nn = 0;
    cudaGraphGetNodes(g, nullptr, &nn);
    std::vector<cudaGraphNode_t> nodes(nn);
    if (nn) cudaGraphGetNodes(g, nodes.data(), &nn);
    long long nk = 0;
    for (size_t q = 0; q < nn; q++) {
      cudaGraphNodeType t;
      if (cudaGraphNodeGetType(nodes[q], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) nk++;
    }
    if ((int)c->graph_kernels.size() < (int)c->graphs.size()) c->graph_kernels.resize(c->graphs.size(), 0);
    c->graph_kernels[mlvl] = nk;
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaGraphInstantiate");
  }
  if (!c->ev0) {
    CK(cudaEventCreate(&c->ev0));
    CK(cudaEventCreate(&c->ev1));
  }
  CK(cudaEventRecord(c->ev0, c->stream));
  CK(cudaGraphLaunch(c->graphs[mlvl], c->stream));
  c->launches += c->graph_kernels[mlvl];
  CK(cudaEventRecord(c->ev1, c->stream));
  return MGE_OK;
}

// residual bookkeeping of solver.f90:160-181 after a cycle at FMG level mlvl
static int read_cycle_residual(mge_ctx* c, int mlvl, int ncyc, double* max_res, double* ini_res) {
  auto& fin = c->lv[mlvl - 1];
  for (size_t q = 0; q < fin.size() && q < 64; q++)
    CK(cudaMemcpyAsync(c->h_rt + q, fin[q].rt_cur, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaGetLastError());
  int rc = check_err(c);
  if (rc) return rc;
  double mr = 1000.0;
  for (size_t q = 0; q < fin.size() && q < 64; q++) {
    double r = c->h_rt[q];
    if ((int)fin[q].rtrms.size() <= ncyc) fin[q].rtrms.resize(ncyc + 1, 0.0);
    fin[q].rtrms[ncyc] = r;
    if (ncyc == 1 && ini_res) *ini_res = r;
    if (r < mr) mr = r;
    if (r != r) return fail(c, MGE_ENAN, "NaN residual (solver.f90:180)");
  }
  *max_res = mr;
  return MGE_OK;
}

int mge_cycle(mge_ctx* c, int mlvl, int ncyc, double* max_res) {
  if (!c || !c->committed || mlvl < 1 || mlvl > (int)c->lv.size() || !max_res) return MGE_EBADCFG;
  CK(cudaSetDevice(c->device));
  int rc = launch_cycle_graph(c, mlvl);
  if (rc) return rc;
  rc = read_cycle_residual(c, mlvl, ncyc, max_res, nullptr);
  if (rc) return rc;
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  c->last_cycle_ms = ms;
  return MGE_OK;
}

double mge_last_cycle_ms(const mge_ctx* c) { return c ? c->last_cycle_ms : 0.0; }

// ------------------------------------------------ asynchronous cycles (many cases in flight)
int mge_cycle_async(mge_ctx* c, int mlvl) {
  if (!c || !c->committed || mlvl < 1 || mlvl > (int)c->lv.size()) return MGE_EBADCFG;
  if (c->pending_mlvl) return fail(c, MGE_EBADCFG, "cycle_async: a cycle is already in flight");
  CK(cudaSetDevice(c->device));
  int rc = launch_cycle_graph(c, mlvl);
  if (rc) return rc;
  auto& fin = c->lv[mlvl - 1];
  for (size_t q = 0; q < fin.size() && q < 64; q++)
    CK(cudaMemcpyAsync(c->h_rt + q, fin[q].rt_cur, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpyAsync(c->h_err, c->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  if (!c->ev_done) CK(cudaEventCreateWithFlags(&c->ev_done, cudaEventDisableTiming));
  CK(cudaEventRecord(c->ev_done, c->stream));
  c->pending_mlvl = mlvl;
  return MGE_OK;
}

int mge_cycle_poll(mge_ctx* c, int ncyc, double* max_res) {
  if (!c || !c->pending_mlvl || !max_res) return MGE_EBADCFG;
  CK(cudaSetDevice(c->device));
  cudaError_t e = cudaEventQuery(c->ev_done);
  if (e == cudaErrorNotReady) return 1;
  if (e != cudaSuccess) return cuda_fail(c, e, "cycle_poll");
  const int mlvl = c->pending_mlvl;
  c->pending_mlvl = 0;
  unsigned w = *c->h_err;
  if (w) {
    cudaMemset(c->d_err, 0, sizeof(unsigned));
    if (w & ERR_NEGPRESS) return fail(c, MGE_ENEGPRESS, "timestep: negative or NaN c^2 (timestep.f90:45-48)");
    if (w & ERR_ZERORHO) return fail(c, MGE_EZERORHO, "efluxb: zero density at a cut cell (efluxb.f90:61-64)");
    if (w & ERR_NAN) return fail(c, MGE_ENAN, "bc_cutcell: wsol is NaN (bc_cutcell.f90:147-156)");
    if (w & ERR_NANRES) return fail(c, MGE_ENAN, "NaN residual (solver.f90:180)");
  }
  auto& fin = c->lv[mlvl - 1];
  double mr = 1000.0;
  for (size_t q = 0; q < fin.size() && q < 64; q++) {
    double r = c->h_rt[q];
    if (ncyc >= 0) {
      if ((int)fin[q].rtrms.size() <= ncyc) fin[q].rtrms.resize(ncyc + 1, 0.0);
      fin[q].rtrms[ncyc] = r;
    }
    if (r < mr) mr = r;
    if (r != r) return fail(c, MGE_ENAN, "NaN residual (solver.f90:180)");
  }
  *max_res = mr;
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, c->ev0, c->ev1) == cudaSuccess) c->last_cycle_ms = ms;
  return MGE_OK;
}

int mge_prolong_async(mge_ctx* c, int mlvl) {
  if (!c || !c->committed || mlvl < 1 || mlvl >= (int)c->lv.size()) return MGE_EBADCFG;
  if (c->pending_mlvl) return fail(c, MGE_EBADCFG, "prolong_async: a cycle is in flight");
  CK(cudaSetDevice(c->device));
  enqueue_movfin(c, mlvl + 1, mlvl);  // FMG prolongation, solver.f90:256-259
  CK(cudaGetLastError());
  return MGE_OK;
}

int mge_device_mem(int device, size_t* free_bytes, size_t* total_bytes) {
  int prev = 0;
  if (cudaGetDevice(&prev) != cudaSuccess) return MGE_ECUDA;
  if (cudaSetDevice(device) != cudaSuccess) return MGE_ECUDA;
  size_t f = 0, t = 0;
  cudaError_t e = cudaMemGetInfo(&f, &t);
  cudaSetDevice(prev);
  if (e != cudaSuccess) return MGE_ECUDA;
  if (free_bytes) *free_bytes = f;
  if (total_bytes) *total_bytes = t;
  return MGE_OK;
}

int mge_set_coop_ctas(mge_ctx* c, int max_ctas) {
  if (!c) return MGE_EBADCFG;
  c->coop_max_ctas = max_ctas < 0 ? 0 : max_ctas;
  for (cudaGraphExec_t& g : c->graphs)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  return MGE_OK;
}

int mge_coop_trace(mge_ctx* c, int level, double* us_out, int nout) {
  Block* bp = getb(c, level, 1);
  if (!bp || !c->committed || !us_out || nout < 1) return MGE_EBADCFG;
  CK(cudaSetDevice(c->device));
  unsigned long long* d = nullptr;
  CK(cudaMalloc(&d, 256 * sizeof(unsigned long long)));
  CK(cudaMemset(d, 0, 256 * sizeof(unsigned long long)));
  bool keep = bp->use_coop;
  bp->use_coop = true;
  c->coop_trace = d;
  enqueue_euler(c, *bp, level, level, false, false, 0, true, true);
  c->coop_trace = nullptr;
  bp->use_coop = keep;
  CK(cudaStreamSynchronize(c->stream));
  unsigned long long h[256];
  cudaError_t e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail(c, e, "coop trace");
  int n = (int)h[255];
  for (int q = 0; q < nout; q++) us_out[q] = (q < n) ? (double)(h[1 + q] - h[q]) * 1e-3 : 0.0;
  return n;
}

long long mge_launch_count(const mge_ctx* c) { return c ? c->launches : 0; }

int mge_kernel_times(mge_ctx* c, int level, int reps, double* ms_out, int nout) {
  Block* bp = getb(c, level, 1);
  if (!bp || !c->committed || reps < 1 || !ms_out) return MGE_EBADCFG;
  CK(cudaSetDevice(c->device));
  Block& b = *bp;
  const mge_params& P = c->prm;
  const int NK = 11;
  // per stage: prep, face and combine pass times (the stages differ in the
  // work the passes do)
  double tot[NK] = {0}, stage_ms[3][MGE_MAX_STAGE] = {};
  int cnt[NK] = {0};
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  auto timed = [&](int kind, auto&& fn) -> int {
    CK(cudaEventRecord(e0, c->stream));
    fn();
    CK(cudaEventRecord(e1, c->stream));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    tot[kind] += ms;
    cnt[kind] += 1;
    return MGE_OK;
  };
  int rc = MGE_OK;
  for (int r = 0; r < reps && !rc; r++) {
    rc = timed(0, [&] { enqueue_timestep(c, b); });
    with_dev(b, [&](auto& D) {
      using T = typename std::remove_reference_t<decltype(D)>::value_type;
      launch_save_wn<T>(D, c->stream);
    });
    for (int m = 1; m <= P.mstage && !rc; m++) {
      StageArgs A;
      std::memset(&A, 0, sizeof(A));
      A.m = m;
      A.fn = P.cstp[m - 1] * P.cfl;
      A.cd = P.cdis[m - 1];
      A.dissip_on = P.cdis[m - 1] > 0.0;
      A.scale_fw = m > 1;
      A.forcing = 0;
      A.first_forcing = 0;
      A.lres = 0;
      A.irs = (m % 2 != 0) && P.smoo > 0.0;
      A.vt = P.vt;
      A.fast = b.fast;
      for (int part = 0; part < 4 && !rc; part++) {
        const double before = tot[1 + part];
        rc = timed(1 + part, [&] {
          with_dev(b, [&](auto& D) {
            using T = typename std::remove_reference_t<decltype(D)>::value_type;
            launch_stage_part<T>(part, D, c->P, A, c->d_err, c->stream);
          });
        });
        if (part != 2) stage_ms[part == 3 ? 2 : part][m - 1] += tot[1 + part] - before;
      }
      if (A.irs)
        for (int part = 0; part < 3 && !rc; part++)
          rc = timed(5 + part, [&] {
            with_dev(b, [&](auto& D) {
              using T = typename std::remove_reference_t<decltype(D)>::value_type;
              launch_irs_part<T>(part, D, c->P, b.tabs, c->stream, b.aux32, b.irs_var, &A);
            });
          });
      if (!rc) rc = timed(8, [&] { enqueue_simple(c, b, 4); });
      if (!rc) rc = timed(9, [&] { enqueue_simple(c, b, 2); });
    }
    if (!rc)
      rc = timed(10, [&] {
        with_dev(b, [&](auto& D) {
          using T = typename std::remove_reference_t<decltype(D)>::value_type;
          launch_rtrms<T>(D, c->P, P.vt, b.rt_partial, b.npart, b.rt_cur, c->stream);
        });
      });
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  for (int q = 0; q < NK && q < nout; q++) ms_out[q] = cnt[q] ? tot[q] / cnt[q] : 0.0;
  // [NK, NK+mstage): face pass per stage; then prep per stage; then combine per stage
  const int order[3] = {1, 0, 2};
  for (int q = 0; q < 3; q++)
    for (int m = 0; m < P.mstage && NK + q * P.mstage + m < nout; m++)
      ms_out[NK + q * P.mstage + m] = stage_ms[order[q]][m] / reps;
  return check_err(c);
}

// solver.f90:109-292 with one CUDA graph per FMG level
int mge_solve(mge_ctx* c, const mge_solve_opts* o, double* hist, int hist_len, int* cycles_done, mge_forces* forces) {
  if (!c || !c->committed) return MGE_EBADCFG;
  CK(cudaSetDevice(c->device));
  const mge_params& P = c->prm;
  const int nlevel = (int)c->lv.size();
  const bool use_graph = o ? o->use_graph != 0 : true;
  int nfin = 0, rc;
  double ini_res = 1.0, max_res = 0.0;
  for (int mlvl = 1; mlvl <= nlevel; mlvl++) {
    for (int ncyc = 1; ncyc <= P.mcyc[mlvl - 1]; ncyc++) {
      if (use_graph) {
        if ((rc = launch_cycle_graph(c, mlvl))) return rc;
      } else {
        enqueue_cycle(c, mlvl);
      }
      if ((rc = read_cycle_residual(c, mlvl, ncyc, &max_res, &ini_res))) return rc;
      if (mlvl == nlevel) {
        if (hist && nfin < hist_len) hist[nfin] = max_res;
        nfin++;
        // mixed form: FP32 coarse corrections stall near an eps32-sized residual
        // drop; refine to FP64 once the drop reaches refine_drop
        if (c->prm.precision == MGE_PREC_MIXED && o && o->refine_drop > 0.0 && max_res <= o->refine_drop * ini_res)
          if ((rc = mge_set_precision(c, MGE_PREC_REFINED))) return rc;
      }
      if (mlvl > 1) {  // convergence (solver.f90:237-239); the single-grid level runs all its cycles
        double drop = P.conv_drop > 0.0 ? P.conv_drop : 1.0e6;
        if (ini_res / max_res > drop) break;
      }
      if (o && o->max_cycles_total > 0 && mlvl == nlevel && nfin >= o->max_cycles_total) break;
    }
    if (mlvl < nlevel) {  // FMG prolongation (solver.f90:256-259)
      enqueue_movfin(c, mlvl + 1, mlvl);
      CK(cudaGetLastError());
      if ((rc = check_err(c))) return rc;
    }
  }
  if (cycles_done) *cycles_done = nfin;
  if (forces) return mge_forces_compute(c, nlevel, o, forces);
  return MGE_OK;
}

size_t mge_device_bytes(const mge_ctx* c) { return c ? c->bytes : 0; }

int mge_sync(mge_ctx* c) {
  if (!c) return MGE_EBADCFG;
  CK(cudaSetDevice(c->device));
  return check_err(c);
}

}  // extern "C"

// ================================================================ groups of cases in lockstep
// Many cases (one context each) advance one multigrid cycle together: every
// phase of the cycle runs as one launch over the block of that level of
// every case (mge_kernels.cu, multi_*), whatever the cases' sizes, and the
// whole lockstep cycle is one captured CUDA graph.  Each case runs the same
// bodies in the same order as its own per-phase path, so its results are
// those it would have alone.
namespace {

struct GroupPlan {
  std::vector<mge_ctx*> cases;
  std::vector<std::pair<unsigned long long, unsigned>> key;  // (uid, gen) per case
  int mlvl = 0, device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, done = nullptr;
  std::vector<MultiLevel> lv;  // per level
  std::vector<MultiPair> pr;   // pr[l]: level l+1 (coarse) and l+2 (fine), 0-based l
  std::vector<void*> allocs;
  cudaGraphExec_t graph = nullptr;
  long long graph_kernels = 0;
  double* d_res = nullptr;     // gathered residuals of the cycle (one per case)
  unsigned* d_errs = nullptr;  // gathered error words
  double* h_res = nullptr;     // pinned
  unsigned* h_errs = nullptr;  // pinned
  unsigned long long last_use = 0;
};

std::mutex g_group_mu;
std::vector<GroupPlan*> g_plans;
unsigned long long g_plan_clock = 0;
constexpr size_t kMaxPlans = 24;

void destroy_plan(GroupPlan* G) {
  cudaSetDevice(G->device);
  if (G->stream) cudaStreamSynchronize(G->stream);
  if (G->graph) cudaGraphExecDestroy(G->graph);
  for (void* p : G->allocs) cudaFree(p);
  if (G->h_res) cudaFreeHost(G->h_res);
  if (G->h_errs) cudaFreeHost(G->h_errs);
  if (G->ev0) cudaEventDestroy(G->ev0);
  if (G->ev1) cudaEventDestroy(G->ev1);
  if (G->done) cudaEventDestroy(G->done);
  if (G->stream) cudaStreamDestroy(G->stream);
  delete G;
}

template <typename T>
int plan_upload(GroupPlan* G, T** dst, const std::vector<T>& v, std::string& why) {
  void* p = nullptr;
  if (cudaMalloc(&p, std::max<size_t>(v.size(), 1) * sizeof(T)) != cudaSuccess) {
    cudaGetLastError();
    why = "group: cudaMalloc";
    return MGE_ENOMEM;
  }
  G->allocs.push_back(p);
  if (!v.empty() && cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) {
    why = "group: cudaMemcpy";
    return MGE_ECUDA;
  }
  *dst = (T*)p;
  return MGE_OK;
}

// item counts of one case's block for each kind (MultiKind)
void kind_counts(const Block& b, long long* n) {
  const long long nx = b.nx, ny = b.ny, nz = b.nz;
  n[MK_PHYS] = nx * ny * nz;
  n[MK_PREP] = (nx + 2) * (ny + 2) * (nz + 2);
  n[MK_FACE] = (nx + 1) * (ny + 1) * (nz + 1);
  n[MK_N] = b.N;
  n[MK_N5] = 5 * b.N;
  n[MK_REC] = (long long)b.recs.size();
  n[MK_IRS0] = 5 * ny * nz;
  n[MK_IRS1] = 5 * nx * nz;
  n[MK_IRS2] = 5 * nx * ny;
  n[MK_BC] = 2 * ((long long)(b.jb + 1) * (b.kb + 1) + (long long)(b.ib + 1) * (b.kb + 1) +
                  (long long)(b.ib + 1) * (b.jb + 1));
  n[MK_CORNER0] = 4LL * (b.kl - 1) + 4LL * (b.jl - 1);
  n[MK_CORNER1] = 4LL * (b.ib + 1);
  n[MK_CORNER2] = 8;
  n[MK_RTP] = 256LL * b.npart;
  n[MK_ONE] = 1;
}

// prefix sums of counts rounded up to whole 256-thread blocks
std::vector<long long> offsets(const std::vector<long long>& cnt) {
  std::vector<long long> off(cnt.size() + 1, 0);
  for (size_t q = 0; q < cnt.size(); q++) off[q + 1] = off[q] + (cnt[q] + 255) / 256 * 256;
  return off;
}

// a plan for the cases, or an error (the cases cannot run in lockstep)
int build_plan(mge_ctx* const* cs, int n, int mlvl, GroupPlan** out, std::string& why) {
  mge_ctx* c0 = cs[0];
  const mge_params& P0 = c0->prm;
  const int nl = (int)c0->lv.size();
  for (int q = 0; q < n; q++) {
    const mge_ctx* c = cs[q];
    const mge_params& P = c->prm;
    if (!c->committed || c->device != c0->device) return why = "group: a case is not committed on this device", MGE_EBADCFG;
    if ((int)c->lv.size() != nl || P.mstage != P0.mstage || P.mgtype != P0.mgtype || P.vt != P0.vt ||
        P.cfl != P0.cfl || P.smoo != P0.smoo || P.irs_variant != 0 || P.execmode != 0 ||
        P.distype != MGE_DIS_CENTRAL || P.eqntype != P0.eqntype || P.dissip != P0.dissip)
      return why = "group: the cases' schedules or schemes differ", MGE_EBADCFG;
    for (int m = 0; m < P.mstage; m++)
      if (P.cstp[m] != P0.cstp[m] || P.cdis[m] != P0.cdis[m]) return why = "group: stage coefficients differ", MGE_EBADCFG;
    for (int l = 0; l < nl; l++) {
      if (c->lv[l].size() != 1) return why = "group: one block per level only", MGE_EBADCFG;
      const Block& b = c->lv[l][0];
      const Block& b0 = c0->lv[l][0];
      if (b.f32 != b0.f32 || b.aux32 != b0.aux32 || b.fast != b0.fast)
        return why = "group: the cases' precision forms differ", MGE_EBADCFG;
    }
    for (int r = 0; r < q; r++)
      if (cs[r] == c) return why = "group: a case appears twice", MGE_EBADCFG;
  }
  GroupPlan* G = new GroupPlan();
  G->cases.assign(cs, cs + n);
  for (int q = 0; q < n; q++) G->key.push_back({cs[q]->uid, cs[q]->gen});
  G->mlvl = mlvl;
  G->device = c0->device;
  int rc = MGE_OK;
  auto bad = [&](int code) {
    destroy_plan(G);
    return code;
  };
  if (cudaStreamCreateWithFlags(&G->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&G->ev0) != cudaSuccess || cudaEventCreate(&G->ev1) != cudaSuccess ||
      cudaEventCreateWithFlags(&G->done, cudaEventDisableTiming) != cudaSuccess)
    return why = "group: stream or events", bad(MGE_ECUDA);
  G->lv.resize(nl);
  for (int l = 0; l < nl; l++) {
    MultiLevel& L = G->lv[l];
    const Block& b0 = c0->lv[l][0];
    L.nc = n;
    L.f32 = b0.f32;
    L.aux32 = b0.aux32;
    L.fast = b0.fast;
    std::vector<DevBlock<double>> bd;
    std::vector<DevBlock<float>> bf;
    std::vector<PhysParams> pp;
    std::vector<unsigned*> er;
    std::vector<IrsTables> tb;
    std::vector<double*> rp, ro;
    std::vector<int> np;
    std::vector<std::vector<long long>> cnt(MK_COUNT, std::vector<long long>(n));
    for (int q = 0; q < n; q++) {
      Block& b = cs[q]->lv[l][0];
      if (b.f32)
        bf.push_back(b.dev32);
      else
        bd.push_back(b.dev);
      pp.push_back(cs[q]->P);
      er.push_back(cs[q]->d_err);
      for (int d = 0; d < 3; d++) tb.push_back(b.tabs[d]);
      rp.push_back(b.rt_partial);
      ro.push_back(b.rt_cur);
      np.push_back(b.npart);
      long long k[MK_COUNT];
      kind_counts(b, k);
      for (int m = 0; m < MK_COUNT; m++) cnt[m][q] = k[m];
    }
    if (L.f32)
      rc = plan_upload(G, (DevBlock<float>**)&L.B, bf, why);
    else
      rc = plan_upload(G, (DevBlock<double>**)&L.B, bd, why);
    if (!rc) rc = plan_upload(G, &L.P, pp, why);
    if (!rc) rc = plan_upload(G, &L.err, er, why);
    if (!rc) rc = plan_upload(G, &L.tab, tb, why);
    if (!rc) rc = plan_upload(G, &L.rt_partial, rp, why);
    if (!rc) rc = plan_upload(G, &L.npart, np, why);
    if (!rc) rc = plan_upload(G, &L.rt_out, ro, why);
    for (int m = 0; m < MK_COUNT && !rc; m++) {
      std::vector<long long> off = offsets(cnt[m]);
      L.tot[m] = off.back();
      rc = plan_upload(G, &L.off[m], off, why);
    }
    if (rc) return bad(rc);
    // small levels: the whole update of every case as one persistent
    // cooperative launch (MGE_GROUP_COOP_MAX_CELLS: the group's cells up to
    // which it does; 300,000 by default)
    long long coop_max = 300000;
    if (const char* e = getenv("MGE_GROUP_COOP_MAX_CELLS")) coop_max = atoll(e);
    L.coop = L.tot[MK_PREP] <= coop_max;
  }
  G->pr.resize(nl > 1 ? nl - 1 : 0);
  for (int l = 0; l + 1 < nl; l++) {
    MultiPair& M = G->pr[l];
    M.nc = n;
    M.c32 = G->lv[l].f32;
    M.f32 = G->lv[l + 1].f32;
    std::vector<DevBlock<double>> cd, fd;
    std::vector<DevBlock<float>> cf, ff;
    std::vector<unsigned char> xs(n * xfer_size());
    std::vector<uint8_t*> mk;
    std::vector<double*> dc;
    std::vector<PhysParams> pp;
    std::vector<std::vector<long long>> cnt(MP_COUNT, std::vector<long long>(n));
    for (int q = 0; q < n; q++) {
      Block& bc = cs[q]->lv[l][0];
      Block& bf_ = cs[q]->lv[l + 1][0];
      if (bf_.parent != 1) return why = "group: a fine block's parent is not the level's block", bad(MGE_EBADCFG);
      if (bc.f32) cf.push_back(bc.dev32); else cd.push_back(bc.dev);
      if (bf_.f32) ff.push_back(bf_.dev32); else fd.push_back(bf_.dev);
      make_xfer_host(bf_.ratio, bf_.offset, xs.data() + q * xfer_size());
      mk.push_back(bc.marker);
      dc.push_back(cs[q]->scratch);
      pp.push_back(cs[q]->P);
      cnt[MP_COLLC][q] = (long long)(bf_.nx / bf_.ratio[0]) * (bf_.ny / bf_.ratio[1]) * (bf_.nz / bf_.ratio[2]);
      cnt[MP_CN][q] = bc.N;
      cnt[MP_FPHYS][q] = (long long)bf_.nx * bf_.ny * bf_.nz;
      cnt[MP_FN][q] = bf_.N;
    }
    if (M.c32) rc = plan_upload(G, (DevBlock<float>**)&M.C, cf, why);
    else rc = plan_upload(G, (DevBlock<double>**)&M.C, cd, why);
    if (!rc) {
      if (M.f32) rc = plan_upload(G, (DevBlock<float>**)&M.F, ff, why);
      else rc = plan_upload(G, (DevBlock<double>**)&M.F, fd, why);
    }
    if (!rc) rc = plan_upload(G, (unsigned char**)&M.X, xs, why);
    if (!rc) rc = plan_upload(G, &M.marker, mk, why);
    if (!rc) rc = plan_upload(G, &M.dc, dc, why);
    if (!rc) rc = plan_upload(G, &M.P, pp, why);
    for (int m = 0; m < MP_COUNT && !rc; m++) {
      std::vector<long long> off = offsets(cnt[m]);
      M.tot[m] = off.back();
      rc = plan_upload(G, &M.off[m], off, why);
    }
    if (rc) return bad(rc);
  }
  std::vector<double> z(n, 0.0);
  std::vector<unsigned> ze(n, 0u);
  if ((rc = plan_upload(G, &G->d_res, z, why)) || (rc = plan_upload(G, &G->d_errs, ze, why))) return bad(rc);
  if (cudaMallocHost(&G->h_res, n * sizeof(double)) != cudaSuccess ||
      cudaMallocHost(&G->h_errs, n * sizeof(unsigned)) != cudaSuccess)
    return why = "group: pinned buffers", bad(MGE_ENOMEM);
  *out = G;
  return MGE_OK;
}

// euler on level `level` of every case (enqueue_euler's per-phase path)
void group_euler(GroupPlan& G, int level, int mgl, int mlvl, bool lres, bool lfir, bool rt, bool with_timestep) {
  const mge_params& P = G.cases[0]->prm;
  StageArgs A[MGE_MAX_STAGE];
  for (int m = 1; m <= P.mstage; m++) {
    A[m - 1] = stage_args(P, m, mgl, mlvl, lres, lfir, 0);
    A[m - 1].fast = G.lv[level - 1].fast;
  }
  multi_euler(G.lv[level - 1], A, P.mstage, with_timestep, lfir, rt && !lres, G.stream);
}

// solver.f90:127-234 for the group: enqueue_cycle with one launch per phase for all cases
void enqueue_group_cycle(GroupPlan& G) {
  const mge_params& P = G.cases[0]->prm;
  const int mlvl = G.mlvl;
  std::vector<int> icyc(G.lv.size() + 2, 0);
  int mgl = mlvl;
  for (;;) {    // lopmg
    for (;;) {  // lopr
      icyc[mgl] += 1;
      const bool lfir = (mgl != mlvl);
      group_euler(G, mgl, mgl, mlvl, false, lfir, mgl == mlvl, true);
      if (mlvl == 1) return;
      group_euler(G, mgl, mgl, mlvl, true, false, false, false);
      mgl = mgl - 1;
      multi_movco_level(G.lv[mgl - 1], &G.pr[mgl - 1], G.stream);
      if (mgl == 1) break;
    }
    bool lfir = true;
    for (;;) {  // lopp
      group_euler(G, mgl, mgl, mlvl, false, lfir, false, true);
      lfir = false;
      mgl = mgl + 1;
      multi_movfin_level(G.lv[mgl - 1], G.pr[mgl - 2], mgl - 1 == mlvl, G.stream);
      if (mgl == mlvl) return;
      if (icyc[mgl] != P.mgtype) break;
      icyc[mgl] = 0;
    }
  }
}

void drop_group_plans(const mge_ctx* c) {
  std::lock_guard<std::mutex> lk(g_group_mu);
  for (size_t q = 0; q < g_plans.size();) {
    GroupPlan* G = g_plans[q];
    if (std::find(G->cases.begin(), G->cases.end(), c) != G->cases.end()) {
      g_plans.erase(g_plans.begin() + q);
      destroy_plan(G);
    } else {
      q++;
    }
  }
}

GroupPlan* find_plan(mge_ctx* const* cs, int n, int mlvl) {
  for (GroupPlan* G : g_plans) {
    if (G->mlvl != mlvl || (int)G->cases.size() != n) continue;
    bool same = true;
    for (int q = 0; q < n && same; q++)
      same = G->cases[q] == cs[q] && G->key[q].first == cs[q]->uid && G->key[q].second == cs[q]->gen;
    if (same) return G;
  }
  return nullptr;
}

}  // namespace

extern "C" {

int mge_group_cycle_async(mge_ctx* const* cases, int n, int mlvl) {
  if (!cases || n < 1) return MGE_EBADCFG;
  for (int q = 0; q < n; q++)
    if (!cases[q] || cases[q]->pending_mlvl || cases[q]->group_pending || mlvl < 1 ||
        mlvl > (int)cases[q]->lv.size())
      return MGE_EBADCFG;
  mge_ctx* c = cases[0];
  CK(cudaSetDevice(c->device));
  std::lock_guard<std::mutex> lk(g_group_mu);
  GroupPlan* G = find_plan(cases, n, mlvl);
  if (!G) {
    std::string why;
    int rc = build_plan(cases, n, mlvl, &G, why);
    if (rc) return fail(c, rc, why);
    if (g_plans.size() >= kMaxPlans) {  // drop the least recently used plan with no cycle in flight
      GroupPlan* old = nullptr;
      for (GroupPlan* P : g_plans) {
        bool busy = false;
        for (mge_ctx* c : P->cases) busy = busy || c->group_pending == P;
        if (!busy && (!old || P->last_use < old->last_use)) old = P;
      }
      if (old) {
        g_plans.erase(std::find(g_plans.begin(), g_plans.end(), old));
        destroy_plan(old);
      }
    }
    g_plans.push_back(G);
  }
  G->last_use = ++g_plan_clock;
  if (!G->graph) {
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(G->stream, cudaStreamCaptureModeThreadLocal));
    enqueue_group_cycle(*G);
    gather_residuals(G->lv[mlvl - 1], G->d_res, G->d_errs, G->stream);
    cudaError_t e = cudaStreamEndCapture(G->stream, &g);
    if (e != cudaSuccess) return cuda_fail(c, e, "group: cudaStreamEndCapture");
    e = cudaGraphInstantiate(&G->graph, g, 0);
    size_t nn = 0;
    cudaGraphGetNodes(g, nullptr, &nn);
    G->graph_kernels = (long long)nn;
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(c, e, "group: cudaGraphInstantiate");
  }
  // the cases' own streams first, the group cycle, then the cases' streams wait for it
  for (int q = 0; q < n; q++) {
    if (!cases[q]->ev_group) CK(cudaEventCreateWithFlags(&cases[q]->ev_group, cudaEventDisableTiming));
    CK(cudaEventRecord(cases[q]->ev_group, cases[q]->stream));
    CK(cudaStreamWaitEvent(G->stream, cases[q]->ev_group, 0));
  }
  CK(cudaEventRecord(G->ev0, G->stream));
  CK(cudaGraphLaunch(G->graph, G->stream));
  CK(cudaEventRecord(G->ev1, G->stream));
  CK(cudaMemcpyAsync(G->h_res, G->d_res, n * sizeof(double), cudaMemcpyDeviceToHost, G->stream));
  CK(cudaMemcpyAsync(G->h_errs, G->d_errs, n * sizeof(unsigned), cudaMemcpyDeviceToHost, G->stream));
  CK(cudaEventRecord(G->done, G->stream));
  for (int q = 0; q < n; q++) {
    CK(cudaStreamWaitEvent(cases[q]->stream, G->done, 0));
    cases[q]->group_pending = G;
    cases[q]->launches += G->graph_kernels;
  }
  return MGE_OK;
}

// 1 while the group's cycle runs; then 0, with each case's finest residual in
// max_res[q] and its stop (0 or an MGE_ code) in rc_out[q]
int mge_group_cycle_poll(mge_ctx* const* cases, int n, int ncyc, double* max_res, int* rc_out) {
  if (!cases || n < 1 || !max_res || !rc_out) return MGE_EBADCFG;
  GroupPlan* G = (GroupPlan*)cases[0]->group_pending;
  if (!G || (int)G->cases.size() != n) return MGE_EBADCFG;
  for (int q = 0; q < n; q++)
    if (cases[q] != G->cases[q] || cases[q]->group_pending != G) return MGE_EBADCFG;
  mge_ctx* c = cases[0];
  CK(cudaSetDevice(c->device));
  cudaError_t e = cudaEventQuery(G->done);
  if (e == cudaErrorNotReady) return 1;
  if (e != cudaSuccess) return cuda_fail(c, e, "group_cycle_poll");
  float ms = 0.f;
  cudaEventElapsedTime(&ms, G->ev0, G->ev1);
  for (int q = 0; q < n; q++) {
    mge_ctx* cq = cases[q];
    cq->group_pending = nullptr;
    cq->last_cycle_ms = ms;
    const unsigned w = G->h_errs[q];
    const double r = G->h_res[q];
    rc_out[q] = MGE_OK;
    if (w) {
      cudaMemsetAsync(cq->d_err, 0, sizeof(unsigned), cq->stream);
      rc_out[q] = (w & ERR_NEGPRESS) ? fail(cq, MGE_ENEGPRESS, "timestep: negative or NaN c^2 (timestep.f90:45-48)")
                  : (w & ERR_ZERORHO) ? fail(cq, MGE_EZERORHO, "efluxb: zero density at a cut cell (efluxb.f90:61-64)")
                  : (w & ERR_NAN)     ? fail(cq, MGE_ENAN, "bc_cutcell: wsol is NaN (bc_cutcell.f90:147-156)")
                                      : fail(cq, MGE_ENAN, "NaN residual (solver.f90:180)");
    } else if (r != r) {
      rc_out[q] = fail(cq, MGE_ENAN, "NaN residual (solver.f90:180)");
    }
    auto& fin = cq->lv[G->mlvl - 1];
    if (ncyc >= 0) {
      if ((int)fin[0].rtrms.size() <= ncyc) fin[0].rtrms.resize(ncyc + 1, 0.0);
      fin[0].rtrms[ncyc] = r;
    }
    max_res[q] = r;
  }
  return MGE_OK;
}

}  // extern "C"
