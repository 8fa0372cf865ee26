// mge_internal.h -- device data model shared by the kernels and the host
// runtime of the GB300 multigrid Runge-Kutta cycle.
//
// Layout of every per-cell field is the reference's Fortran layout
// a(0:ib,0:jb,0:kb,nvar): cell (i,j,k) at c = i + Pi*(j + Pj*k), variable v
// at v*N + c.  Per-cell flux/face scratch uses [dir][var][N].
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mge {

// One uniform block as the kernels see it (passed by value).
template <typename T>
struct DevBlock {
  typedef T value_type;
  int nx, ny, nz;
  int il, jl, kl, ie, je, ke, ib, jb, kb;
  int Pi, Pj;
  long long N;              // (ib+1)(jb+1)(kb+1)
  // state and stage fields (precision T)
  T* w;                     // 5N conservative variables
  T* p;                     // N pressure
  T* wn;                    // 5N state at the start of euler
  T* w1;                    // 5N state of the previous physical time step (unsteady only, else null)
  T* w2;                    // 5N state of the one before
  T* ws;                    // 5N state saved on first coarse entry
  T* dw;                    // 5N residual
  T* fw;                    // 5N blended dissipation
  T* wr;                    // 5N restricted residual (coarse levels)
  T* qf;                    // 5N multigrid forcing
  T* vdtim;                 // N local time step
  T* lam;                   // N radi+radj+radk
  double* dtim;             // 1 global time step (FP64 bits, atomicMin target)
  const uint8_t* blank;     // N
  const uint8_t* marker;    // N
  const int32_t* cutmap;    // N: -1 or cut-target index
  // per-stage scratch shared by the blocks of a context
  T* H;                     // N  rho*E + p
  T* F;                     // 15N per-cell convective flux [dir][var]
  T* fp;                    // 3N pressure sensor [dir]
  T* efs;                   // 15N convective face flux [dir][var] at the upper cell of the face
  T* dfs;                   // 15N dissipative face flux
  T* dlt;                   // 15N differences w(q)-w(q-1) along each direction [dir][var], enthalpy in var 5
  T* vt;                    // 4N velocity and temperature (Navier-Stokes)
  T* vfs;                   // 15N viscous face flux (Navier-Stokes)
  T* eps;                   // 3N smoothing coefficients eps_x,y,z (psmoo variant only, else null)
  // metric (uniform, axis-aligned face vectors)
  double s[3];              // si[0], sj[1], sk[2]
  double hx, hy, hz;        // cell sizes (viscous gradients)
  double rh[3], r4h[3];     // RN(1/h) and RN(1/(4h)) per axis, for FP64 blocks
  float rhf[3], r4hf[3];    // the same in single precision, of the single-precision h
  double sqrt_ds[3];        // sqrt(s*s) computed on the host
  double vol;
  double rvol;              // RN(1/vol)
  float rvolf;              // RN(1/vol) in single precision, of the single-precision vol
  // cut-cell records
  int nmir;
  int m0;                   // first record with an empty cloud (nmir if none)
  const int32_t* rec_i;     // [nmir][8]: ccid(3), faceid, zz, npoint, counted in the forces, pad
  const int32_t* rec_cloud; // [nmir][8][3]
  const double* rec_coef;   // [nmir][8]
  const double* rec_nvec;   // [nmir][3]
  const double* rec_qb;     // [nmir][3]
  const double* rec_area;   // [nmir] wall-face area
  T* rec_wsol;              // [nmir][5]
  T* rec_psol;              // [nmir]
  T* rec_wall;              // [nmir][25] wall-side terms of the current stage (rec_wall_terms)
  const int32_t* tgt_off;   // [ntgt+1]
  const int32_t* tgt_ops;   // op = 2*m + role (0: cut cell, 1: neighbour)
  int bctype[6];
  double fnv[6][3];
};

struct StageArgs {
  int m;            // stage 1..mstage
  double fn;        // cstp(m)*cfl
  double cd;        // cdis(m)
  int dissip_on;    // cdis(m) > 0
  int scale_fw;     // m > 1
  int forcing;      // mgl < mlvl
  int first_forcing;// lfir && m == 1
  int lres;
  int irs;          // odd stage with smoo > 0: defer the update to the line sweeps
  int vt;
  int tmode;        // unsteady source term: 0 none, 1 first step (itime 1), 2 BDF2 (itime > 1)
  int fast;         // the contracted FP64 residual of the mixed form's finest level (JST central, Euler)
};

struct PhysParams {
  double gamma, gm1, gm;    // gamma, gamma-1, 1/(gamma-1)
  double vis2, vis4, cfl, dimcfl;
  double rho0, p0, c0, u0[3];
  double e0;                // rho0*h0 - p0
  double si_far;            // rho0**gamma/p0
  int matrix;               // matrix dissipation
  int eqn_ns;
  double smoo;
  int vt;                   // global time step
  int distype;              // MGE_DIS_* (0 central, 1 Roe first order, 2 Roe MUSCL)
  int irs_kind;             // 0 psmoo_old (what euler calls), 1 psmoo + progon3
  int gamma14;              // gamma is 1.4: the far field's powers take the short forms of fast_pow.cuh
  double pow_dg, pow_dm;    // gamma - 7/5 and 1/(gamma-1) - 5/2 (the double exponents' offsets)
  int unsteady;             // execmode 1: dual time stepping
  double dtstep;            // physical time step
  double viscl, kt, gas_const, prlmean;  // laminar viscosity, heat conductivity, R, Pr
  double cfac;              // viscous weight of the time step (timestep.f90:119-125)
  double epsentr;           // Harten entropy fix
  double lim_e2[5];         // van Albada floor per primitive variable
  double rgm1;              // RN(1/(gamma-1))
  float rgm1f;              // RN(1/(gamma-1)) in single precision, of the single-precision gamma-1
  double rgamma;            // RN(1/gamma)
  float rgammaf;            // RN(1/gamma) in single precision, of the single-precision gamma
};

// error word: the kernels set it only while it is zero (atomicCAS), so it
// holds the first stop in launch order, the one the reference's sequential
// run would have stopped at
enum : unsigned {
  ERR_NEGPRESS = 1u,
  ERR_ZERORHO = 2u,
  ERR_NAN = 4u,
  ERR_NANRES = 8u,  // NaN residual norm (solver.f90:180)
};

// IRS pivot tables of one block direction (psmoo.f90:136-166)
struct IrsTables {
  const double* e1;   // pivot of row q (index 0..l)
  const double* e1r;  // RN(1/pivot)
  const double* e2;   // elimination factor
  // the same in single precision for the FP32 sweeps: the rounded pivot, the
  // single-precision RN(1/pivot) of that rounded pivot, the rounded factor
  const float* e1f;
  const float* e1rf;
  const float* e2f;
};

// one euler update as a single cooperative launch (small grids)
struct EulerLaunch {
  int mstage, do_timestep, lfir, lres, rt;
  StageArgs st[8];
  IrsTables tab[3];
  double* rt_partial;
  int npart;
  double* rt_out;
  unsigned* err;
  unsigned long long* trace;  // optional phase timestamps (profiling hook)
  int max_ctas;               // cap on the cooperative grid (0: occupancy limit)
};

// ---------------------------------------------------------------- several cases per launch
// The same phase of a group of cases (one block per case: the blocks of one
// level) in one launch.  Item kinds: the count of work items one case has
// for a phase; every case's range is rounded up to whole 256-thread blocks.
enum MultiKind {
  MK_PHYS = 0,   // physical cells nx*ny*nz
  MK_PREP,       // [1..ie]^3
  MK_FACE,       // [2..ie]^3
  MK_N,          // all cells N
  MK_N5,         // 5N
  MK_REC,        // cut-cell records
  MK_IRS0,       // 5 * lines along i, j, k
  MK_IRS1,
  MK_IRS2,
  MK_BC,         // boundary-pass items
  MK_CORNER0,    // corner phases
  MK_CORNER1,
  MK_CORNER2,
  MK_RTP,        // 256 * residual partial sums
  MK_ONE,        // one thread block
  MK_COUNT
};

// device arrays of one level of a group (built by the runtime)
struct MultiLevel {
  int nc = 0;
  bool f32 = false, aux32 = false, fast = false;
  bool coop = false;             // the update as one persistent cooperative launch (k_group_euler)
  void* B = nullptr;             // DevBlock<T>[nc]
  PhysParams* P = nullptr;       // [nc]
  unsigned** err = nullptr;      // [nc]
  IrsTables* tab = nullptr;      // [3 nc]
  double** rt_partial = nullptr; // [nc]
  int* npart = nullptr;          // [nc]
  double** rt_out = nullptr;     // [nc]
  long long* off[MK_COUNT] = {};  // [nc + 1] per kind
  long long tot[MK_COUNT] = {};
};

// the transfer between two levels of a group: child block f of each case and
// its parent c on the level above
enum MultiPairKind { MP_COLLC = 0, MP_CN, MP_FPHYS, MP_FN, MP_COUNT };
struct MultiPair {
  int nc = 0;
  bool c32 = false, f32 = false;
  void* C = nullptr;             // DevBlock<TC>[nc]
  void* F = nullptr;             // DevBlock<TF>[nc]
  void* X = nullptr;             // Xfer[nc]
  uint8_t** marker = nullptr;    // [nc] the parents' markers
  double** dc = nullptr;         // [nc] the cases' stage scratch
  PhysParams* P = nullptr;       // [nc]
  long long* off[MP_COUNT] = {};
  long long tot[MP_COUNT] = {};
};

// the lockstep steps of the group cycle (mge_kernels.cu)
void multi_euler(const MultiLevel& L, const StageArgs* A, int mstage, bool with_timestep, bool lfir, bool rt,
                 cudaStream_t s);
void multi_movco_level(const MultiLevel& L, const MultiPair* pair, cudaStream_t s);
void multi_movfin_level(const MultiLevel& L, const MultiPair& pair, bool fmg, cudaStream_t s);
void gather_residuals(const MultiLevel& L, double* res, unsigned* errs, cudaStream_t s);
size_t xfer_size();
void make_xfer_host(const int ratio[3], const int offset[3], void* out);

// kernel launchers (mge_kernels.cu)
template <typename T> int launch_euler_coop(const DevBlock<T>& b, const PhysParams& P, const EulerLaunch& L, int device,
                                            cudaStream_t s, bool aux32 = false);
template <typename T> void launch_timestep(const DevBlock<T>& b, const PhysParams& P, unsigned* err, cudaStream_t s,
                                           bool aux32 = false);
template <typename T> void launch_stage(const DevBlock<T>& b, const PhysParams& P, const StageArgs& A, unsigned* err,
                                        cudaStream_t s, cudaStream_t side = nullptr, cudaEvent_t fork = nullptr,
                                        cudaEvent_t join = nullptr);
template <typename T> void launch_irs(const DevBlock<T>& b, const PhysParams& P, const IrsTables* tab, cudaStream_t s,
                                      bool aux32 = false, const int* variant = nullptr,
                                      const StageArgs* A = nullptr);
template <typename T> void launch_stage_part(int part, const DevBlock<T>& b, const PhysParams& P, const StageArgs& A,
                                             unsigned* err, cudaStream_t s);
template <typename T> void launch_irs_part(int part, const DevBlock<T>& b, const PhysParams& P, const IrsTables* tab,
                                           cudaStream_t s, bool aux32 = false, const int* variant = nullptr,
                                           const StageArgs* A = nullptr);
template <typename T> void launch_solut(const DevBlock<T>& b, const PhysParams& P, double rm, double p_tot, int ns,
                                        double* out, cudaStream_t s);
template <typename T> void launch_cutcell(const DevBlock<T>& b, const PhysParams& P, unsigned* err, cudaStream_t s);
template <typename T> void launch_bcond(const DevBlock<T>& b, const PhysParams& P, cudaStream_t s);
template <typename T> void launch_rtrms(const DevBlock<T>& b, const PhysParams& P, int vt, double* partial,
                                        int npartial, double* out, cudaStream_t s, unsigned* err = nullptr);
template <typename T> void launch_depvars_all(const DevBlock<T>& b, const PhysParams& P, cudaStream_t s);
template <typename T> void launch_copy_ws(const DevBlock<T>& b, cudaStream_t s);
template <typename T> void launch_save_wn(const DevBlock<T>& b, cudaStream_t s);
template <typename T> void launch_copy_wn(const DevBlock<T>& b, cudaStream_t s);
template <typename T> void launch_init_free(const DevBlock<T>& b, const PhysParams& P, cudaStream_t s);
template <typename TC, typename TF>
void launch_collc(const DevBlock<TC>& c, const DevBlock<TF>& f, const int ratio[3], const int offset[3],
                  uint8_t* marker_c, cudaStream_t s);
template <typename TF, typename TC>
void launch_addw(const DevBlock<TF>& f, const DevBlock<TC>& c, const int ratio[3], const int offset[3], int fmg,
                 double* scratch, cudaStream_t s);
template <typename TF, typename TC>
void launch_embed(const DevBlock<TF>& f, const DevBlock<TC>& c, const int ratio[3], const int offset[3],
                  const PhysParams& P, cudaStream_t s);
template <typename T> void launch_forces(const DevBlock<T>& b, const double* origin, const double* h,
                                         const double* center, double mu, double* out7, cudaStream_t s);
template <typename T>
void launch_overlap(const DevBlock<T>& g, const DevBlock<T>& p, const long long* dst, const long long* src,
                    const double* fac, long long n, const PhysParams& P, cudaStream_t s);
int rtrms_partials(long long ncells);
void init_kernel_attributes();
void launch_convert(const void* src, bool src32, void* dst, bool dst32, long long n, cudaStream_t s);
// movsurf.f90:31 and bc_cutcell.f90:50 over nmir records: pnew = psurf + pnew
// (pnew holds the displacements on entry), qb = qb / vel_fs (qb holds the
// wall velocities on entry)
void launch_movsurf(long long nmir, const double* psurf, double* pnew, double* qb, double vel_fs, cudaStream_t s);

}  // namespace mge
