// TEST INFRASTRUCTURE -- the CPU oracle.  Only tests/, __graft_entry__.smoke()
// and bench.py's cpu_baseline / reference legs load this library, and only as
// the checker or the timed CPU baseline; the product never links it.
//
// FP64 restatement of the reference's per-timestep spectral core
// (KhaledGhannam/LES, Fortran 90, rprec = kind(1.d0), types.f90:6), routine by
// routine and in the reference's evaluation order, on the reference's array
// layout: real fields (ld,ny,nz) column-major, complex planes (lh,ny) over the
// same storage, pressure (ld,ny,0:nz).  Non-MPI build (nproc = 1, lbz = 1),
// lbc_mom = 'wall', lbc = 1, ifilter = 1 (spectral cutoff), filter_size = 1,
// molec = dns_bc = use_bldg = inflow = .false., ubc = 0, no Coriolis; the
// humidity qmix (scalars_module_q.f90) is advanced when q_flag = 1 and is
// identically zero otherwise.
//
// Parity status: the reference cannot be compiled here (no Fortran compiler,
// no FFTW 2) and ships no tests or golden vectors, so this restatement is
// pinned by known-answer tests (spectral derivatives of trigonometric fields,
// exact 3/2-rule products, tridiagonal vs dense solves, filter transfer
// functions, exact trilinear interpolation of linear fields, divergence-free
// projection) and by its FFT matching numpy.fft: parity is pinned by these
// properties, not by outputs of the reference program itself.
//
// Deliberate, documented deviations (all at the rounding level or in values
// nothing reads):
//  * x**(-1/8) in lagrange_Sdep.f90:324,365 and lagrange_Ssim.f90:259 is
//    evaluated as 1/sqrt(sqrt(sqrt(x))) (correctly rounded operations only),
//    so that CPU and GPU see identical bits before the FP32 truncation that
//    follows in lagrange_Sdep.
//  * the padding columns ld-1:ld hold zeros after a complex-to-real transform
//    (FFTW leaves unspecified values there); what reads them: the plane sums
//    of scaledep_dynamic (scaledep_dynamic.f90:187-243) and std_dynamic
//    (std_dynamic.f90:130-132), taken over 1:nx here, and lagrange_Ssim's
//    relaxation of the padding columns (LM = MM = 0 there).
//  * scaledep_dynamic is called with its own 7-argument interface; the
//    reference's call site (sgs_stag.f90:132) passes 10 arguments.
//  * surface inputs are given nondimensional (zo) and kinematic (wt_s [K m/s],
//    wq_s [g/kg m/s]) instead of being read from zom.dat / wts.dat / wqs.dat
//    [W/m^2] (bottombc.f90:31-59).
//  * thermo (atm_thermodynamics.f90:37-52) fills columns 1..nx and leaves the
//    padding columns zero (the reference evaluates its formulas on whatever
//    the padding holds; nothing reads those values).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>
#include <algorithm>
#include <map>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle_fft.h"
#include "../include/les_gb300.h"

namespace les_oracle {

static const double PI = 3.1415926535897932384626433;  // param.f90:51
static const double BOGUS = -1234567890.0;             // param.f90:50
static const double TADV1 = 1.5, TADV2 = 1.0 - 1.5;    // param.f90:151

using Field = std::vector<double>;

struct Oracle {
  les_config cfg;
  int nx, ny, nz, ld, lh, nx2, ny2, ld_big, lh_big;
  double dx, dy, dz, L_x, L_y, z_i, u_star, dt, vonk, T_scale, dTdz_top, Pr, g, q_scale, dqdz_top;
  int cs_count, model;
  bool s_flag, initu, initsc, q_flag;
  int jt = 0, jt_total = 0;
  double tt = 0.0;
  std::unique_ptr<FFT2> fs, fb;

  size_t nplane, nfield, nplane_big;
  // sim_param.f90:18-38
  Field u, v, w, theta;
  Field dudx, dudy, dudz, dvdx, dvdy, dvdz, dwdx, dwdy, dwdz;
  Field RHSx, RHSy, RHSz, RHSx_f, RHSy_f, RHSz_f;
  Field dpdx, dpdy, dpdz;
  Field txx, txy, tyy, txz, tyz, tzz;
  Field p;  // 0:nz
  Field divtx, divty, divtz;
  // sgsmodule.f90:8-34
  Field F_LM, F_MM, F_QN, F_NN, Beta, Cs_opt2, Nu_t, u_lag, v_lag, w_lag;
  // model 7: G_LM..G_NN, Pr_t, u_lag_s.. (sgsmodule.f90:8-34), TnLMMM, TnQNNN
  Field G_LM, G_MM, G_QN, G_NN, Pr_t, u_lag_s, v_lag_s, w_lag_s, TnLMMM, TnQNNN;
  Field S11, S12, S13, S22, S23, S33;
  // scalars_module.f90:31-36
  Field beta_scal, dTdx, dTdy, dTdz, RHS_T, RHS_Tf;
  // scalars_module_q.f90:17-27
  Field qmix, dqdx, dqdy, dqdz, RHS_q, RHS_qf;
  // bottombc.f90:9-16 (nx,ny)
  Field zo, z_os, wt_s, ustar_avg, phi_m, psi_m, psi_m0, phi_h, psi_h, psi_h0, sgs_t3;
  Field wq_s, sgs_q3;  // bottombc.f90:15, scalars_module_q.f90:23 (level 1)
  // the whole vertical SGS flux arrays sgs_t3, sgs_q3 (ld,ny,nz) of
  // scalar_RHS_calc (level 1 the surface flux), read by MM_XYZ_Out
  Field sgs_t3_vol, sgs_q3_vol;
  // io.f90:403-1218 MM_XYZ_Out running statistics, (nx,ny,nz-1) each
  std::vector<Field> stats;
  std::vector<std::string> stat_names;
  int stats_c = 0, stats_p = 0;
  // fft.f90:19, test_filtermodule.f90:9
  Field kx, ky, k2, G_test, G_test_test;
  double rmsdiv_last = 0.0;
  Field Beta_avg, Betaclip_avg;

  // indexing, Fortran 1-based
  inline size_t I(int jx, int jy, int jz) const {
    return (size_t)(jx - 1) + (size_t)ld * ((size_t)(jy - 1) + (size_t)ny * (size_t)(jz - 1));
  }
  inline size_t P(int jx, int jy, int jz) const {  // p(ld,ny,0:nz)
    return (size_t)(jx - 1) + (size_t)ld * ((size_t)(jy - 1) + (size_t)ny * (size_t)jz);
  }
  inline size_t S2(int jx, int jy) const { return (size_t)(jx - 1) + (size_t)nx * (jy - 1); }
  inline size_t K(int jx, int jy) const { return (size_t)(jx - 1) + (size_t)lh * (jy - 1); }
  double* lev(Field& f, int jz) { return f.data() + (size_t)(jz - 1) * nplane; }

  explicit Oracle(const les_config& c) : cfg(c) {
    nx = c.nx; ny = c.ny; nz = c.nz;
    nx2 = 3 * nx / 2; ny2 = 3 * ny / 2;                // param.f90:59
    lh = nx / 2 + 1; ld = 2 * lh; lh_big = nx2 / 2 + 1; ld_big = 2 * lh_big;  // :60
    L_x = c.l_x; L_y = c.l_y; z_i = c.z_i;
    dz = (c.lz_over_zi * z_i) / z_i / (nz - 1);        // param.f90:64
    dx = L_x / nx; dy = L_y / ny;                      // param.f90:65
    u_star = c.u_star; dt = c.dt; vonk = c.vonk; T_scale = c.t_scale;
    dTdz_top = c.dtdz_top; Pr = c.pr; g = c.g;
    q_flag = c.q_flag != 0; q_scale = c.q_scale; dqdz_top = c.dqdz_top;
    cs_count = c.cs_count; model = c.model;
    s_flag = c.s_flag != 0; initu = c.initu != 0; initsc = c.initsc != 0;
    jt_total = c.jt_total0;
    fs.reset(new FFT2(nx, ny));
    fb.reset(new FFT2(nx2, ny2));
    nplane = (size_t)ld * ny; nfield = nplane * nz; nplane_big = (size_t)ld_big * ny2;
    Field* fl[] = {&u, &v, &w, &theta, &dudx, &dudy, &dudz, &dvdx, &dvdy, &dvdz, &dwdx, &dwdy,
                   &dwdz, &RHSx, &RHSy, &RHSz, &RHSx_f, &RHSy_f, &RHSz_f, &dpdx, &dpdy, &dpdz,
                   &txx, &txy, &tyy, &txz, &tyz, &tzz, &divtx, &divty, &divtz, &F_LM, &F_MM,
                   &F_QN, &F_NN, &Beta, &Cs_opt2, &Nu_t, &u_lag, &v_lag, &w_lag, &S11, &S12,
                   &S13, &S22, &S23, &S33, &beta_scal, &dTdx, &dTdy, &dTdz, &RHS_T, &RHS_Tf,
                   &qmix, &dqdx, &dqdy, &dqdz, &RHS_q, &RHS_qf, &sgs_t3_vol, &sgs_q3_vol,
                   &G_LM, &G_MM, &G_QN, &G_NN, &Pr_t, &u_lag_s, &v_lag_s, &w_lag_s, &TnLMMM, &TnQNNN};
    for (Field* f : fl) f->assign(nfield, 0.0);
    p.assign(nplane * (nz + 1), 0.0);
    Field* sf[] = {&zo, &z_os, &wt_s, &ustar_avg, &phi_m, &psi_m, &psi_m0, &phi_h, &psi_h,
                   &psi_h0, &sgs_t3, &wq_s, &sgs_q3};
    for (Field* f : sf) f->assign((size_t)nx * ny, 0.0);
    for (double& x : phi_m) x = 1.0;
    for (double& x : Pr_t) x = Pr;  // the reference reads Pr_t from the restart record
    for (double& x : phi_h) x = 1.0;
    Beta_avg.assign(nz, 0.0); Betaclip_avg.assign(nz, 0.0);
    init_wavenumber();
    G_test.assign((size_t)lh * ny, 0.0); G_test_test.assign((size_t)lh * ny, 0.0);
    test_filter_init(2.0 * 1.0, G_test);   // main.f90:166, filter_size = 1
    test_filter_init(4.0 * 1.0, G_test_test);  // main.f90:169
  }

  // fft.f90:54-81
  void init_wavenumber() {
    kx.assign((size_t)lh * ny, 0.0); ky.assign((size_t)lh * ny, 0.0); k2.assign((size_t)lh * ny, 0.0);
    for (int jx = 1; jx <= lh - 1; ++jx)
      for (int jy = 1; jy <= ny; ++jy) kx[K(jx, jy)] = (double)(jx - 1);
    for (int jy = 1; jy <= ny; ++jy) {
      int m = ((jy - 1 + ny / 2) % ny + ny) % ny - ny / 2;
      for (int jx = 1; jx <= lh; ++jx) ky[K(jx, jy)] = (double)m;
    }
    for (int jy = 1; jy <= ny; ++jy) { kx[K(lh, jy)] = 0.0; ky[K(lh, jy)] = 0.0; }
    for (int jx = 1; jx <= lh; ++jx) { kx[K(jx, ny / 2 + 1)] = 0.0; ky[K(jx, ny / 2 + 1)] = 0.0; }
    const double fx = 2.0 * PI / L_x, fy = 2.0 * PI / L_y;
    for (size_t i = 0; i < kx.size(); ++i) {
      kx[i] = fx * kx[i];
      ky[i] = fy * ky[i];
      k2[i] = kx[i] * kx[i] + ky[i] * ky[i];
    }
  }

  // test_filtermodule.f90:32-63 (ifilter = 1)
  void test_filter_init(double alpha, Field& G) {
    const double norm = 1.0 / (double)(nx * ny);
    for (double& x : G) x = norm;
    const double delta = alpha * std::sqrt(dx * dy);
    const double q = PI / delta;
    const double kc2 = q * q;
    for (size_t i = 0; i < G.size(); ++i)
      if (k2[i] >= kc2) G[i] = 0.0;
    for (int jy = 1; jy <= ny; ++jy) G[K(lh, jy)] = 0.0;
    for (int jx = 1; jx <= lh; ++jx) G[K(jx, ny / 2 + 1)] = 0.0;
  }

  // ---- complex-plane helpers (lh,ny) view of an (ld,ny) plane -----------
  static inline double& RE(double* pl, int ld_, int jx, int jy) {
    return pl[(size_t)2 * (jx - 1) + (size_t)ld_ * (jy - 1)];
  }
  static inline double& IM(double* pl, int ld_, int jx, int jy) {
    return pl[(size_t)2 * (jx - 1) + 1 + (size_t)ld_ * (jy - 1)];
  }
  void kill_oddballs(double* pl) {  // f(lh,:)=0 ; f(:,ny/2+1)=0
    for (int jy = 1; jy <= ny; ++jy) { RE(pl, ld, lh, jy) = 0.0; IM(pl, ld, lh, jy) = 0.0; }
    for (int jx = 1; jx <= lh; ++jx) {
      RE(pl, ld, jx, ny / 2 + 1) = 0.0; IM(pl, ld, jx, ny / 2 + 1) = 0.0;
    }
  }
  // dst = eye * k * src   (complex (0,k)*(a,b) = (-k b, k a))
  void eye_k(double* dst, const double* src, const Field& k) {
    for (int jy = 1; jy <= ny; ++jy)
      for (int jx = 1; jx <= lh; ++jx) {
        const double kk = k[K(jx, jy)];
        const double a = src[(size_t)2 * (jx - 1) + (size_t)ld * (jy - 1)];
        const double b = src[(size_t)2 * (jx - 1) + 1 + (size_t)ld * (jy - 1)];
        dst[(size_t)2 * (jx - 1) + (size_t)ld * (jy - 1)] = -(kk * b);
        dst[(size_t)2 * (jx - 1) + 1 + (size_t)ld * (jy - 1)] = kk * a;
      }
  }

  // filt_da.f90:3-42, levels 1..nlev
  void filt_da(double* f, double* dfdx, double* dfdy, int nlev) {
    const double c = 1.0 / (double)(nx * ny);
#pragma omp parallel for schedule(static)
    for (int jz = 1; jz <= nlev; ++jz) {
      double* fp = f + (size_t)(jz - 1) * nplane;
      double* xp = dfdx + (size_t)(jz - 1) * nplane;
      double* yp = dfdy + (size_t)(jz - 1) * nplane;
      for (size_t i = 0; i < nplane; ++i) fp[i] = c * fp[i];
      fs->r2c(fp);
      kill_oddballs(fp);
      eye_k(yp, fp, ky);
      eye_k(xp, fp, kx);
      fs->c2r(fp);
      fs->c2r(xp);
      fs->c2r(yp);
    }
  }
  // ddx.f90:1-31 / ddy.f90:1-31
  void ddxy_one(double* df, const double* f, int nlev, const Field& k) {
    const double c = 1.0 / (double)(nx * ny);
#pragma omp parallel for schedule(static)
    for (int jz = 1; jz <= nlev; ++jz) {
      double* dp = df + (size_t)(jz - 1) * nplane;
      const double* fp = f + (size_t)(jz - 1) * nplane;
      for (size_t i = 0; i < nplane; ++i) dp[i] = c * fp[i];
      fs->r2c(dp);
      kill_oddballs(dp);
      eye_k(dp, dp, k);
      fs->c2r(dp);
    }
  }
  void ddx(double* df, const double* f, int nlev) { ddxy_one(df, f, nlev, kx); }
  void ddy(double* df, const double* f, int nlev) { ddxy_one(df, f, nlev, ky); }
  // ddxy.f90:1-29
  void ddxy(double* dfdx, double* dfdy, const double* f, int nlev) {
    const double c = 1.0 / (double)(nx * ny);
#pragma omp parallel for schedule(static)
    for (int jz = 1; jz <= nlev; ++jz) {
      double* xp = dfdx + (size_t)(jz - 1) * nplane;
      double* yp = dfdy + (size_t)(jz - 1) * nplane;
      const double* fp = f + (size_t)(jz - 1) * nplane;
      for (size_t i = 0; i < nplane; ++i) xp[i] = c * fp[i];
      fs->r2c(xp);
      kill_oddballs(xp);
      eye_k(yp, xp, ky);
      eye_k(xp, xp, kx);
      fs->c2r(xp);
      fs->c2r(yp);
    }
  }
  // ddz_uv.f90:5-57 (non-MPI): 2..nz-1, nz = 0, level 1 untouched
  void ddz_uv(double* dfdz, const double* f) {
    const double c = 1.0 / dz;
    for (int jz = 2; jz <= nz - 1; ++jz)
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= nx; ++jx)
          dfdz[I(jx, jy, jz)] = c * (f[I(jx, jy, jz)] - f[I(jx, jy, jz - 1)]);
    for (size_t i = 0; i < nplane; ++i) dfdz[(size_t)(nz - 1) * nplane + i] = 0.0;
  }
  // ddz_w.f90:6-51 (non-MPI): 1..nz-1, nz = 0
  void ddz_w(double* dfdz, const double* f) {
    const double c = 1.0 / dz;
    for (int jz = 1; jz <= nz - 1; ++jz)
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= nx; ++jx)
          dfdz[I(jx, jy, jz)] = c * (f[I(jx, jy, jz + 1)] - f[I(jx, jy, jz)]);
    for (size_t i = 0; i < nplane; ++i) dfdz[(size_t)(nz - 1) * nplane + i] = 0.0;
  }
  // padd.f90:1-26 on one complex plane
  void padd(double* ub, const double* us) {
    std::fill(ub, ub + nplane_big, 0.0);
    for (int jy = 1; jy <= ny / 2; ++jy)
      for (int jx = 1; jx <= nx / 2; ++jx) {
        ub[(size_t)2 * (jx - 1) + (size_t)ld_big * (jy - 1)] = us[(size_t)2 * (jx - 1) + (size_t)ld * (jy - 1)];
        ub[(size_t)2 * (jx - 1) + 1 + (size_t)ld_big * (jy - 1)] = us[(size_t)2 * (jx - 1) + 1 + (size_t)ld * (jy - 1)];
      }
    for (int jy = 1; jy <= ny / 2 - 1; ++jy)
      for (int jx = 1; jx <= nx / 2; ++jx) {
        const int jb = jy + ny2 - ny / 2 + 1, js = jy + ny / 2 + 1;
        ub[(size_t)2 * (jx - 1) + (size_t)ld_big * (jb - 1)] = us[(size_t)2 * (jx - 1) + (size_t)ld * (js - 1)];
        ub[(size_t)2 * (jx - 1) + 1 + (size_t)ld_big * (jb - 1)] = us[(size_t)2 * (jx - 1) + 1 + (size_t)ld * (js - 1)];
      }
  }
  // unpadd.f90:1-22 on one complex plane
  void unpadd(double* cc, const double* cb) {
    for (int jy = 1; jy <= ny / 2; ++jy)
      for (int jx = 1; jx <= nx / 2; ++jx) {
        RE(cc, ld, jx, jy) = cb[(size_t)2 * (jx - 1) + (size_t)ld_big * (jy - 1)];
        IM(cc, ld, jx, jy) = cb[(size_t)2 * (jx - 1) + 1 + (size_t)ld_big * (jy - 1)];
      }
    for (int jy = 1; jy <= ny; ++jy) { RE(cc, ld, nx / 2 + 1, jy) = 0.0; IM(cc, ld, nx / 2 + 1, jy) = 0.0; }
    for (int jx = 1; jx <= lh; ++jx) { RE(cc, ld, jx, ny / 2 + 1) = 0.0; IM(cc, ld, jx, ny / 2 + 1) = 0.0; }
    for (int jy = 1; jy <= ny / 2 - 1; ++jy)
      for (int jx = 1; jx <= nx / 2; ++jx) {
        const int jb = jy + ny2 - ny / 2 + 1, js = jy + ny / 2 + 1;
        RE(cc, ld, jx, js) = cb[(size_t)2 * (jx - 1) + (size_t)ld_big * (jb - 1)];
        IM(cc, ld, jx, js) = cb[(size_t)2 * (jx - 1) + 1 + (size_t)ld_big * (jb - 1)];
      }
  }
  // dealias1.f90:1-31 : u (ld,ny,nlev) -> u_big (ld_big,ny2,nlev)
  void dealias1(const double* uu, double* ub, int nlev) {
    const double c = 1.0 / (double)(nx * ny);
#pragma omp parallel for schedule(static)
    for (int jz = 1; jz <= nlev; ++jz) {
      std::vector<double> temp(nplane);
      const double* up = uu + (size_t)(jz - 1) * nplane;
      for (size_t i = 0; i < nplane; ++i) temp[i] = c * up[i];
      fs->r2c(temp.data());
      double* bp = ub + (size_t)(jz - 1) * nplane_big;
      padd(bp, temp.data());
      fb->c2r(bp);
    }
  }
  // dealias2.f90:1-33 : u_big -> u
  void dealias2(double* uu, double* ub, int nlev) {
    const double c = 1.0 / (double)(nx2 * ny2);
    for (size_t i = 0; i < nplane_big * nlev; ++i) ub[i] = c * ub[i];
#pragma omp parallel for schedule(static)
    for (int jz = 1; jz <= nlev; ++jz) {
      double* bp = ub + (size_t)(jz - 1) * nplane_big;
      double* up = uu + (size_t)(jz - 1) * nplane;
      fb->r2c(bp);
      unpadd(up, bp);
      fs->c2r(up);
    }
  }
  // test_filtermodule.f90:13-30 : one (ld,ny) plane in place
  void test_filter(double* f, const Field& G) {
    fs->r2c(f);
    for (int jy = 1; jy <= ny; ++jy)
      for (int jx = 1; jx <= lh; ++jx) {
        const double gg = G[K(jx, jy)];
        RE(f, ld, jx, jy) = gg * RE(f, ld, jx, jy);
        IM(f, ld, jx, jy) = gg * IM(f, ld, jx, jy);
      }
    fs->c2r(f);
  }

  // convec.f90:1-248
  void convec(double* cx, double* cy, double* cz) {
    std::vector<double> u1b(nplane_big * nz), u2b(nplane_big * nz), u3b(nplane_big * nz);
    std::vector<double> v1b(nplane_big * nz), v2b(nplane_big * nz), v3b(nplane_big * nz);
    std::vector<double> ccb(nplane_big * nz);
    double c = 1.0 / (double)(nx * ny);
#pragma omp parallel for schedule(static)
    for (int jz = 1; jz <= nz; ++jz) {
      double* X = cx + (size_t)(jz - 1) * nplane;
      double* Y = cy + (size_t)(jz - 1) * nplane;
      double* Z = cz + (size_t)(jz - 1) * nplane;
      const size_t o = (size_t)(jz - 1) * nplane;
      for (size_t i = 0; i < nplane; ++i) { X[i] = c * u[o + i]; Y[i] = c * v[o + i]; Z[i] = c * w[o + i]; }
      fs->r2c(X); fs->r2c(Y); fs->r2c(Z);
      const size_t ob = (size_t)(jz - 1) * nplane_big;
      padd(&u1b[ob], X); padd(&u2b[ob], Y); padd(&u3b[ob], Z);
      fb->c2r(&u1b[ob]); fb->c2r(&u2b[ob]); fb->c2r(&u3b[ob]);
    }
#pragma omp parallel for schedule(static)
    for (int jz = 1; jz <= nz; ++jz) {
      double* X = cx + (size_t)(jz - 1) * nplane;
      double* Y = cy + (size_t)(jz - 1) * nplane;
      double* Z = cz + (size_t)(jz - 1) * nplane;
      const size_t o = (size_t)(jz - 1) * nplane;
      if (jz == 1) {  // lbc_mom = 'wall'
        for (size_t i = 0; i < nplane; ++i) {
          X[i] = c * (0.5 * (dwdy[i] + dwdy[nplane + i]) - dvdz[i]);
          Y[i] = c * (dudz[i] - 0.5 * (dwdx[i] + dwdx[nplane + i]));
        }
      } else {
        for (size_t i = 0; i < nplane; ++i) {
          X[i] = c * (dwdy[o + i] - dvdz[o + i]);
          Y[i] = c * (dudz[o + i] - dwdx[o + i]);
        }
      }
      for (size_t i = 0; i < nplane; ++i) Z[i] = c * (dvdx[o + i] - dudy[o + i]);
      fs->r2c(X); fs->r2c(Y); fs->r2c(Z);
      const size_t ob = (size_t)(jz - 1) * nplane_big;
      padd(&v1b[ob], X); padd(&v2b[ob], Y); padd(&v3b[ob], Z);
      fb->c2r(&v1b[ob]); fb->c2r(&v2b[ob]); fb->c2r(&v3b[ob]);
    }
    c = 1.0 / (double)(nx2 * ny2);
    const size_t NB = nplane_big;
    auto B = [&](std::vector<double>& a, int jz, size_t i) -> double { return a[(size_t)(jz - 1) * NB + i]; };
    // CX
    for (size_t i = 0; i < NB; ++i)
      ccb[i] = c * (B(u2b, 1, i) * (-B(v3b, 1, i)) + 0.5 * B(u3b, 2, i) * (B(v2b, 2, i)));
#pragma omp parallel for schedule(static)
    for (int jz = 2; jz <= nz - 1; ++jz)
      for (size_t i = 0; i < NB; ++i)
        ccb[(size_t)(jz - 1) * NB + i] =
            c * (B(u2b, jz, i) * (-B(v3b, jz, i)) +
                 0.5 * (B(u3b, jz + 1, i) * (B(v2b, jz + 1, i)) + B(u3b, jz, i) * (B(v2b, jz, i))));
    back_to_small(ccb.data(), cx);
    // CY
    for (size_t i = 0; i < NB; ++i)
      ccb[i] = c * (B(u1b, 1, i) * (B(v3b, 1, i)) + 0.5 * B(u3b, 2, i) * (-B(v1b, 2, i)));
#pragma omp parallel for schedule(static)
    for (int jz = 2; jz <= nz - 1; ++jz)
      for (size_t i = 0; i < NB; ++i)
        ccb[(size_t)(jz - 1) * NB + i] =
            c * (B(u1b, jz, i) * (B(v3b, jz, i)) +
                 0.5 * (B(u3b, jz + 1, i) * (-B(v1b, jz + 1, i)) + B(u3b, jz, i) * (-B(v1b, jz, i))));
    back_to_small(ccb.data(), cy);
    // CZ
    for (size_t i = 0; i < NB; ++i) ccb[i] = 0.0;
#pragma omp parallel for schedule(static)
    for (int jz = 2; jz <= nz - 1; ++jz)
      for (size_t i = 0; i < NB; ++i)
        ccb[(size_t)(jz - 1) * NB + i] =
            c * 0.5 * ((B(u1b, jz, i) + B(u1b, jz - 1, i)) * (-B(v2b, jz, i)) +
                       (B(u2b, jz, i) + B(u2b, jz - 1, i)) * (B(v1b, jz, i)));
    back_to_small(ccb.data(), cz);
    for (size_t i = 0; i < nplane; ++i) {
      const size_t o = (size_t)(nz - 1) * nplane;
      cx[o + i] = BOGUS; cy[o + i] = BOGUS; cz[o + i] = BOGUS;
    }
  }
  void back_to_small(double* ccb, double* out) {  // convec.f90:144-151
#pragma omp parallel for schedule(static)
    for (int jz = 1; jz <= nz - 1; ++jz) {
      double* bp = ccb + (size_t)(jz - 1) * nplane_big;
      double* op = out + (size_t)(jz - 1) * nplane;
      fb->r2c(bp);
      unpadd(op, bp);
      fs->c2r(op);
    }
  }

  // sgs_stag.f90:371-498 calc_Sij, lbc_mom = 'wall'
  void calc_Sij() {
    for (int jy = 1; jy <= ny; ++jy)
      for (int jx = 1; jx <= nx; ++jx) {
        const size_t i1 = I(jx, jy, 1), i2 = I(jx, jy, 2);
        double ux = dudx[i1], uy = dudy[i1], uz = dudz[i1];
        double vx = dvdx[i1], vy = dvdy[i1], vz = dvdz[i1];
        double wx = 0.5 * (dwdx[i1] + dwdx[i2]);
        double wy = 0.5 * (dwdy[i1] + dwdy[i2]);
        double wz = dwdz[i1];
        S11[i1] = ux; S12[i1] = 0.5 * (uy + vx); S13[i1] = 0.5 * (uz + wx);
        S22[i1] = vy; S23[i1] = 0.5 * (vz + wy); S33[i1] = wz;
      }
    for (int jz = 2; jz <= nz; ++jz)
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= nx; ++jx) {
          const size_t i = I(jx, jy, jz), im = I(jx, jy, jz - 1);
          double ux = 0.5 * (dudx[i] + dudx[im]);
          double uy = 0.5 * (dudy[i] + dudy[im]);
          double uz = dudz[i];
          double vx = 0.5 * (dvdx[i] + dvdx[im]);
          double vy = 0.5 * (dvdy[i] + dvdy[im]);
          double vz = dvdz[i];
          double wx = dwdx[i];
          double wy = dwdy[i];
          double wz = 0.5 * (dwdz[i] + dwdz[im]);
          S11[i] = ux; S12[i] = 0.5 * (uy + vx); S13[i] = 0.5 * (uz + wx);
          S22[i] = vy; S23[i] = 0.5 * (vz + wy); S33[i] = wz;
        }
  }

  static inline double smag(double a11, double a22, double a33, double a12, double a13, double a23) {
    return std::sqrt(2.0 * (a11 * a11 + a22 * a22 + a33 * a33 + 2.0 * (a12 * a12 + a13 * a13 + a23 * a23)));
  }
  static inline double f32(double x) { return (double)(float)x; }
  static inline double fmax32(double a_already_float, double b) {  // max(real(a), real(b))
    float fa = (float)a_already_float, fb = (float)b;
    return (double)(fa > fb ? fa : fb);
  }

  // sgs_stag.f90:3-364
  void sgs_stag() {
    const double delta = 1.0 * std::pow(dx * dy, 1.0 / 2.0);  // :43
    calc_Sij();
    std::vector<double> txzp((size_t)nx * ny), tyzp((size_t)nx * ny);
    for (int jy = 1; jy <= ny; ++jy)
      for (int jx = 1; jx <= nx; ++jx) { txzp[S2(jx, jy)] = txz[I(jx, jy, 1)]; tyzp[S2(jx, jy)] = tyz[I(jx, jy, 1)]; }
    if (model == 4 || model == 5 || model == 7) {  // :59-69
      for (size_t i = 0; i < nfield; ++i) { u_lag[i] += u[i]; v_lag[i] += v[i]; w_lag[i] += w[i]; }
      for (size_t i = 0; i < nfield; ++i) { u_lag_s[i] += u[i]; v_lag_s[i] += v[i]; w_lag_s[i] += w[i]; }
    }
    const double l = delta;  // :109
    if ((jt >= 1 || initu) && (jt % cs_count == 0)) {  // :120-121, DYN_init = 1
      if (model == 2 || model == 3) {  // sgs_stag.f90:124-135
        std::vector<double> ziko(nz);
        if (model == 2)
          std_dynamic(ziko.data(), S11.data(), S12.data(), S13.data(), S22.data(), S23.data(), S33.data());
        else
          scaledep_dynamic(ziko.data(), S11.data(), S12.data(), S13.data(), S22.data(), S23.data(), S33.data());
        for (int jz = 1; jz <= nz; ++jz)
          for (size_t i = 0; i < nplane; ++i) Cs_opt2[(size_t)(jz - 1) * nplane + i] = ziko[jz - 1];
      } else if (model == 4) {  // sgs_stag.f90:136-137
        lagrange_Ssim(S11.data(), S12.data(), S13.data(), S22.data(), S23.data(), S33.data());
      } else if (model == 5) {
        lagrange_Sdep(S11.data(), S12.data(), S13.data(), S22.data(), S23.data(), S33.data());
      } else if (model == 7) {  // :147-149
        lagrange_Sdep(S11.data(), S12.data(), S13.data(), S22.data(), S23.data(), S33.data());
        Field cs2pr(nfield, 0.0);
        lagrange_scalar_Sdep(cs2pr.data(), S11.data(), S12.data(), S13.data(), S22.data(), S23.data(),
                             S33.data());
      }
    }
    if (model == 5 || model == 6 || model == 7) {  // :166-173
      if (jt_total < 500) {
        const float c016 = 0.16f;
        const double cs = (double)(c016 * c016);
        for (double& x : Cs_opt2) x = cs;
        for (double& x : Pr_t) x = Pr;
      }
    }
    for (int jz = 1; jz <= nz; ++jz)  // :179-211
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= nx; ++jx) {
          const size_t i = I(jx, jy, jz);
          double S = smag(S11[i], S22[i], S33[i], S12[i], S13[i], S23[i]);
          Nu_t[i] = S * Cs_opt2[i] * (l * l);
        }
    for (int jy = 1; jy <= ny; ++jy)  // :221-242 'wall'
      for (int jx = 1; jx <= nx; ++jx) {
        const size_t i = I(jx, jy, 1);
        const double cst = Nu_t[i], nu = 0.0;
        txx[i] = -2.0 * (cst + nu) * S11[i];
        txy[i] = -2.0 * (cst + nu) * S12[i];
        tyy[i] = -2.0 * (cst + nu) * S22[i];
        tzz[i] = -2.0 * (cst + nu) * S33[i];
      }
    for (int jz = 2; jz <= nz - 1; ++jz)  // :281-302
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= nx; ++jx) {
          const size_t i = I(jx, jy, jz), ip = I(jx, jy, jz + 1);
          const double cst = 0.5 * (Nu_t[i] + Nu_t[ip]), nu = 0.0;
          txx[i] = -2.0 * (cst + nu) * 0.5 * (S11[i] + S11[ip]);
          txy[i] = -2.0 * (cst + nu) * 0.5 * (S12[i] + S12[ip]);
          tyy[i] = -2.0 * (cst + nu) * 0.5 * (S22[i] + S22[ip]);
          tzz[i] = -2.0 * (cst + nu) * 0.5 * (S33[i] + S33[ip]);
        }
    for (int jz = 2; jz <= nz - 1; ++jz)  // :306-317
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= nx; ++jx) {
          const size_t i = I(jx, jy, jz);
          const double cst = Nu_t[i], nu = 0.0;
          txz[i] = -2.0 * (cst + nu) * S13[i];
          tyz[i] = -2.0 * (cst + nu) * S23[i];
        }
    for (int jy = 1; jy <= ny; ++jy)
      for (int jx = 1; jx <= nx; ++jx) { txz[I(jx, jy, 1)] = txzp[S2(jx, jy)]; tyz[I(jx, jy, 1)] = tyzp[S2(jx, jy)]; }
    const size_t o = (size_t)(nz - 1) * nplane;
    for (size_t i = 0; i < nplane; ++i) {
      txx[o + i] = BOGUS; txy[o + i] = BOGUS; tyy[o + i] = BOGUS; tzz[o + i] = BOGUS;
      txz[o + i] = 0.0; tyz[o + i] = 0.0;
    }
  }

  // interpolag_Sdep.f90:2-380 (non-MPI, read_inflow_file = .false.)
  void interpolag_Sdep() {
    Field* F[4] = {&F_LM, &F_MM, &F_QN, &F_NN};
    interpolag(4, true, F, u_lag, v_lag, w_lag);
  }
  // interpolag_scalar_Sdep.f90:1-227: the same algorithm on G_* along the
  // scalar path's Lagrangian velocity sums
  void interpolag_scalar_Sdep() {
    Field* G[4] = {&G_LM, &G_MM, &G_QN, &G_NN};
    interpolag(4, true, G, u_lag_s, v_lag_s, w_lag_s);
  }
  // interpolag_Ssim.f90:3-316: the same back-trajectory interpolation of
  // F_LM and F_MM only, without the near-wall clip of interpolag_Sdep.f90:
  // 290-293 (its w_lag(1) keeps 0.25 w_lag(2), doubled when positive)
  void interpolag_Ssim() {
    Field* F[4] = {&F_LM, &F_MM, &F_QN, &F_NN};
    interpolag(2, false, F, u_lag, v_lag, w_lag);
  }
  void interpolag(const int nf, const bool sdep_clip, Field* const* Fs, Field& u_lag, Field& v_lag, Field& w_lag) {
    const int NX = nx + 2, NY = ny + 2, NZ = nz + 2;
    std::vector<double> FLM((size_t)NX * NY * NZ), FMM(FLM.size()), FQN(FLM.size()), FNN(FLM.size());
    auto FI = [&](int i, int j, int k) { return (size_t)(i - 1) + (size_t)NX * ((size_t)(j - 1) + (size_t)NY * (k - 1)); };
    std::vector<double>* FF[4] = {&FLM, &FMM, &FQN, &FNN};
    for (int q = 0; q < nf; ++q) {
      std::vector<double>& A = *FF[q];
      const Field& Fq = *Fs[q];
      for (int jz = 1; jz <= nz; ++jz)
        for (int jy = 1; jy <= ny; ++jy)
          for (int jx = 1; jx <= nx; ++jx) A[FI(jx + 1, jy + 1, jz + 1)] = Fq[I(jx, jy, jz)];
      for (int k = 1; k <= NZ; ++k)
        for (int j = 1; j <= NY; ++j) { A[FI(1, j, k)] = A[FI(nx + 1, j, k)]; A[FI(nx + 2, j, k)] = A[FI(2, j, k)]; }
      for (int k = 1; k <= NZ; ++k)
        for (int i = 1; i <= NX; ++i) { A[FI(i, 1, k)] = A[FI(i, ny + 1, k)]; A[FI(i, ny + 2, k)] = A[FI(i, 2, k)]; }
      for (int j = 1; j <= NY; ++j)
        for (int i = 1; i <= NX; ++i) A[FI(i, j, 1)] = A[FI(i, j, 2)];
      for (int j = 1; j <= NY; ++j)
        for (int i = 1; i <= NX; ++i) A[FI(i, j, nz + 2)] = A[FI(i, j, nz + 1)];
    }
    const double cs = (double)cs_count;
    for (size_t i = 0; i < nfield; ++i) { u_lag[i] = u_lag[i] / cs; v_lag[i] = v_lag[i] / cs; }
    for (int jz = nz; jz >= 2; --jz)
      for (size_t i = 0; i < nplane; ++i) {
        const size_t a = (size_t)(jz - 1) * nplane + i, b = (size_t)(jz - 2) * nplane + i;
        u_lag[a] = 0.5 * (u_lag[a] + u_lag[b]);
        v_lag[a] = 0.5 * (v_lag[a] + v_lag[b]);
      }
    for (size_t i = 0; i < nfield; ++i) w_lag[i] = w_lag[i] / cs;
    for (size_t i = 0; i < nplane; ++i) w_lag[i] = 0.25 * w_lag[nplane + i];
    for (size_t i = 0; i < nfield; ++i) {
      u_lag[i] = -u_lag[i] * dt * cs / dx;
      v_lag[i] = -v_lag[i] * dt * cs / dy;
      w_lag[i] = -w_lag[i] * dt * cs / dz;
    }
    for (int jy = 1; jy <= ny; ++jy)
      for (int jx = 1; jx <= nx; ++jx) {
        double& w2 = w_lag[I(jx, jy, 2)];
        double& w1 = w_lag[I(jx, jy, 1)];
        w2 = w2 + std::min(w2, 0.0);
        w1 = w1 + std::max(w1, 0.0);
      }
    if (sdep_clip)
      for (size_t i = 0; i < nplane; ++i) {
        double& w2 = w_lag[nplane + i];
        double& w1 = w_lag[i];
        w2 = std::min(1.0, w2);
        w1 = std::min(1.0, w2);
        w2 = std::max(-1.0, w2);
        w1 = std::max(-1.0, w2);
      }
    for (int jz = 1; jz <= nz; ++jz) {
      const int jjz = jz + 1;
      for (int jy = 1; jy <= ny; ++jy) {
        const int jjy = jy + 1;
        for (int jx = 1; jx <= nx; ++jx) {
          const int jjx = jx + 1;
          const size_t i = I(jx, jy, jz);
          const int addx = std::signbit(u_lag[i]) && u_lag[i] != 0.0 ? -1 : 1;  // sign(1,x), -0 -> +1
          const int addy = std::signbit(v_lag[i]) && v_lag[i] != 0.0 ? -1 : 1;
          const int addz = std::signbit(w_lag[i]) && w_lag[i] != 0.0 ? -1 : 1;
          const int jxa = jjx + addx, jya = jjy + addy, jza = jjz + addz;
          const double comp_x = std::fabs(u_lag[i]), comp_y = std::fabs(v_lag[i]), comp_z = std::fabs(w_lag[i]);
          const double frac_x = 1.0 - comp_x, frac_y = 1.0 - comp_y, frac_z = 1.0 - comp_z;
          for (int q = 0; q < nf; ++q) {
            const std::vector<double>& A = *FF[q];
            (*Fs[q])[i] = frac_x * frac_y * (A[FI(jjx, jjy, jjz)] * frac_z + A[FI(jjx, jjy, jza)] * comp_z) +
                          frac_x * comp_y * (A[FI(jjx, jya, jjz)] * frac_z + A[FI(jjx, jya, jza)] * comp_z) +
                          comp_x * frac_y * (A[FI(jxa, jjy, jjz)] * frac_z + A[FI(jxa, jjy, jza)] * comp_z) +
                          comp_x * comp_y * (A[FI(jxa, jya, jjz)] * frac_z + A[FI(jxa, jya, jza)] * comp_z);
          }
        }
      }
    }
    std::fill(u_lag.begin(), u_lag.end(), 0.0);
    std::fill(v_lag.begin(), v_lag.end(), 0.0);
    std::fill(w_lag.begin(), w_lag.end(), 0.0);
  }

  static inline double pow_m18(double x) { return 1.0 / std::sqrt(std::sqrt(std::sqrt(x))); }

  // lagrange_Ssim.f90:5-335 (model 4; inilag = .false., inflow = .false., no
  // buildings, no level set): Beta = 1 (:122), interpolag_Ssim (:126); per
  // level the G_test filters of std_dynamic with fourbeta = 4 Beta
  // (:140-219), LM and MM per point (:221-222), the Lagrangian relaxation
  // with T = 1.5 delta (F_LM F_MM)^(-1/8) over lagran_dt = cs_count dt
  // (:258-264, x^(-1/8) as 1/sqrt(sqrt(sqrt(x)))), F_LM >= eps (:265),
  // Cs^2 = F_LM / F_MM, 0 on the padding columns, >= eps (:267-269);
  // eps = 1e-32 (:25).
  // The relaxation covers the padding columns too, where LM = MM = 0 (the
  // test-filtered planes are zero there).
  void lagrange_Ssim(const double* s11, const double* s12, const double* s13, const double* s22,
                     const double* s23, const double* s33) {
    const double eps = 1e-32;
    const double delta = 1.0 * std::pow(dx * dy, 1.0 / 2.0);
    const double opftdelta = 1.5 * delta;
    std::fill(Beta.begin(), Beta.end(), 1.0);
    interpolag_Ssim();
    const double lagran_dt = dt * (double)cs_count;
    const double cst = 2.0 * (delta * delta);
#pragma omp parallel for schedule(static)
    for (int jz = 1; jz <= nz; ++jz) {
      const size_t NP = nplane, o = (size_t)(jz - 1) * NP;
      std::vector<double> buf(NP * 21);
      auto pl = [&](int q) { return buf.data() + (size_t)q * NP; };
      for (size_t i = 0; i < NP; ++i) {
        double ub, vb, wb;
        if (jz == 1) {
          ub = u[i]; vb = v[i]; wb = 0.25 * w[NP + i];
        } else {
          ub = 0.5 * (u[o + i] + u[o - NP + i]); vb = 0.5 * (v[o + i] + v[o - NP + i]); wb = w[o + i];
        }
        pl(0)[i] = ub; pl(1)[i] = vb; pl(2)[i] = wb;
        pl(3)[i] = ub * ub; pl(4)[i] = ub * vb; pl(5)[i] = ub * wb;  // :154-159
        pl(6)[i] = vb * vb; pl(7)[i] = vb * wb; pl(8)[i] = wb * wb;
      }
      const int ia[6] = {0, 0, 0, 1, 1, 2}, ib[6] = {0, 1, 2, 1, 2, 2};
      for (int q = 0; q < 3; ++q) test_filter(pl(q), G_test);
      for (int q = 0; q < 6; ++q) {
        test_filter(pl(3 + q), G_test);
        for (size_t i = 0; i < NP; ++i) pl(3 + q)[i] = pl(3 + q)[i] - pl(ia[q])[i] * pl(ib[q])[i];
      }
      const double* Sp[6] = {s11 + o, s12 + o, s13 + o, s22 + o, s23 + o, s33 + o};
      for (size_t i = 0; i < NP; ++i) {
        const double S = smag(Sp[0][i], Sp[3][i], Sp[5][i], Sp[1][i], Sp[2][i], Sp[4][i]);
        for (int q = 0; q < 6; ++q) { pl(9 + q)[i] = Sp[q][i]; pl(15 + q)[i] = S * Sp[q][i]; }
      }
      for (int q = 0; q < 12; ++q) test_filter(pl(9 + q), G_test);
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= ld; ++jx) {
          const size_t i = (size_t)(jx - 1) + (size_t)ld * (jy - 1);
          double LM = 0.0, MM = 0.0;
          if (jx <= nx) {
            double b[6], sb[6], Lq[6], M[6];
            for (int q = 0; q < 6; ++q) { b[q] = pl(9 + q)[i]; sb[q] = pl(15 + q)[i]; Lq[q] = pl(3 + q)[i]; }
            const double Sb = smag(b[0], b[3], b[5], b[1], b[2], b[4]);
            const double fourbeta = 4.0 * Beta[o + i];
            for (int q = 0; q < 6; ++q) M[q] = cst * (sb[q] - fourbeta * Sb * b[q]);
            LM = Lq[0] * M[0] + Lq[3] * M[3] + Lq[5] * M[5] + 2.0 * (Lq[1] * M[1] + Lq[2] * M[2] + Lq[4] * M[4]);
            MM = M[0] * M[0] + M[3] * M[3] + M[5] * M[5] + 2.0 * (M[1] * M[1] + M[2] * M[2] + M[4] * M[4]);
          }
          double& flm = F_LM[o + i];
          double& fmm = F_MM[o + i];
          double Tn = std::max(flm * fmm, eps);
          Tn = opftdelta * pow_m18(Tn);
          const double dumfac = lagran_dt / Tn;
          const double epsi = dumfac / (1.0 + dumfac);
          flm = epsi * LM + (1.0 - epsi) * flm;
          fmm = epsi * MM + (1.0 - epsi) * fmm;
          flm = std::max(eps, flm);
          double cs = flm / fmm;
          if (jx > nx) cs = 0.0;
          Cs_opt2[o + i] = std::max(eps, cs);
        }
    }
  }

  // lagrange_Sdep.f90:4-478 (inilag = .false., inflow = .false.)
  void lagrange_Sdep(const double* s11, const double* s12, const double* s13, const double* s22,
                     const double* s23, const double* s33) {
    const double delta = 1.0 * std::pow(dx * dy, 1.0 / 2.0);
    const double tf1 = 2.0, tf2 = 4.0, tf1_2 = tf1 * tf1, tf2_2 = tf2 * tf2;
    const double opftdelta = 1.5 * delta;
    interpolag_Sdep();
    const double lagran_dt = dt * (double)cs_count;
    const double cst = 2.0 * (delta * delta);
    const double bexp = std::log(tf1) / (std::log(tf2) - std::log(tf1));
    const float f1em24 = 1e-24f;
#pragma omp parallel for schedule(static)
    for (int jz = 1; jz <= nz; ++jz) {
      const size_t NP = nplane;
      std::vector<double> buf(NP * 42);
      auto pl = [&](int q) { return buf.data() + (size_t)q * NP; };
      // 0..2 u_bar v_bar w_bar ; 3..5 u_hat v_hat w_hat ; 6..11 L ; 12..17 Q
      // 18..23 S_bar ; 24..29 S_hat ; 30..35 S_S_bar ; 36..41 S_S_hat
      const size_t o = (size_t)(jz - 1) * NP;
      for (size_t i = 0; i < NP; ++i) {
        double ub, vb, wb;
        if (jz == 1) { ub = u[i]; vb = v[i]; wb = 0.25 * w[NP + i]; }
        else {
          ub = 0.5 * (u[o + i] + u[o - NP + i]);
          vb = 0.5 * (v[o + i] + v[o - NP + i]);
          wb = w[o + i];
        }
        pl(0)[i] = ub; pl(1)[i] = vb; pl(2)[i] = wb;
        pl(3)[i] = ub; pl(4)[i] = vb; pl(5)[i] = wb;
        pl(6)[i] = ub * ub; pl(7)[i] = ub * vb; pl(8)[i] = ub * wb;
        pl(9)[i] = vb * vb; pl(10)[i] = vb * wb; pl(11)[i] = wb * wb;
        for (int q = 0; q < 6; ++q) pl(12 + q)[i] = pl(6 + q)[i];
      }
      for (int q = 0; q < 3; ++q) test_filter(pl(q), G_test);
      const int ia[6] = {0, 0, 0, 1, 1, 2}, ib[6] = {0, 1, 2, 1, 2, 2};
      for (int q = 0; q < 6; ++q) {
        test_filter(pl(6 + q), G_test);
        for (size_t i = 0; i < NP; ++i) pl(6 + q)[i] = pl(6 + q)[i] - pl(ia[q])[i] * pl(ib[q])[i];
      }
      for (int q = 0; q < 3; ++q) test_filter(pl(3 + q), G_test_test);
      for (int q = 0; q < 6; ++q) {
        test_filter(pl(12 + q), G_test_test);
        for (size_t i = 0; i < NP; ++i) pl(12 + q)[i] = pl(12 + q)[i] - pl(3 + ia[q])[i] * pl(3 + ib[q])[i];
      }
      const double* Sp[6] = {s11 + o, s12 + o, s13 + o, s22 + o, s23 + o, s33 + o};
      std::vector<double> S(NP);
      for (size_t i = 0; i < NP; ++i) {
        S[i] = smag(Sp[0][i], Sp[3][i], Sp[5][i], Sp[1][i], Sp[2][i], Sp[4][i]);
        for (int q = 0; q < 6; ++q) {
          pl(18 + q)[i] = Sp[q][i];
          pl(24 + q)[i] = Sp[q][i];
          pl(30 + q)[i] = S[i] * Sp[q][i];
          pl(36 + q)[i] = S[i] * Sp[q][i];
        }
      }
      for (int q = 0; q < 6; ++q) test_filter(pl(18 + q), G_test);
      for (int q = 0; q < 6; ++q) test_filter(pl(24 + q), G_test_test);
      for (int q = 0; q < 6; ++q) test_filter(pl(30 + q), G_test);
      for (int q = 0; q < 6; ++q) test_filter(pl(36 + q), G_test_test);
      // order of the six components: 11 12 13 22 23 33
      double sum2d = 0.0, sumcs = 0.0, sum4d = 0.0;
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= nx; ++jx) {
          const size_t i = (size_t)(jx - 1) + (size_t)ld * (jy - 1);
          const size_t gi = o + i;
          double Sb = smag(pl(18)[i], pl(21)[i], pl(23)[i], pl(19)[i], pl(20)[i], pl(22)[i]);
          double Sh = smag(pl(24)[i], pl(27)[i], pl(29)[i], pl(25)[i], pl(26)[i], pl(28)[i]);
          double M[6], N[6];
          for (int q = 0; q < 6; ++q) {
            M[q] = cst * (pl(30 + q)[i] - tf1_2 * Sb * pl(18 + q)[i]);
            N[q] = cst * (pl(36 + q)[i] - tf2_2 * Sh * pl(24 + q)[i]);
          }
          const double* L = nullptr;
          double Lq[6], Qq[6];
          for (int q = 0; q < 6; ++q) { Lq[q] = pl(6 + q)[i]; Qq[q] = pl(12 + q)[i]; }
          (void)L;
          // LM = L11*M11+L22*M22+L33*M33+2*(L12*M12+L13*M13+L23*M23)  (:282-285)
          double LM = Lq[0] * M[0] + Lq[3] * M[3] + Lq[5] * M[5] + 2.0 * (Lq[1] * M[1] + Lq[2] * M[2] + Lq[4] * M[4]);
          double MM = M[0] * M[0] + M[3] * M[3] + M[5] * M[5] + 2.0 * (M[1] * M[1] + M[2] * M[2] + M[4] * M[4]);
          double QN = Qq[0] * N[0] + Qq[3] * N[3] + Qq[5] * N[5] + 2.0 * (Qq[1] * N[1] + Qq[2] * N[2] + Qq[4] * N[4]);
          double NN = N[0] * N[0] + N[3] * N[3] + N[5] * N[5] + 2.0 * (N[1] * N[1] + N[2] * N[2] + N[4] * N[4]);
          // :321-331
          double Tn = fmax32(F_LM[gi] * F_MM[gi], (double)f1em24);
          TnLMMM[gi] = Tn;  // :322
          Tn = opftdelta * pow_m18(Tn);
          Tn = fmax32((double)f1em24, Tn);
          double dumfac = lagran_dt / Tn;
          double epsi = dumfac / (1.0 + dumfac);
          F_LM[gi] = (epsi * LM + (1.0 - epsi) * F_LM[gi]);
          F_MM[gi] = (epsi * MM + (1.0 - epsi) * F_MM[gi]);
          F_LM[gi] = fmax32((double)f1em24, F_LM[gi]);
          double cs2d = F_LM[gi] / F_MM[gi];
          cs2d = fmax32((double)f1em24, cs2d);
          // :362-385
          Tn = fmax32(F_QN[gi] * F_NN[gi], (double)f1em24);
          TnQNNN[gi] = Tn;  // :363
          Tn = opftdelta * pow_m18(Tn);
          Tn = fmax32((double)f1em24, Tn);
          dumfac = lagran_dt / Tn;
          epsi = dumfac / (1.0 + dumfac);
          F_QN[gi] = (epsi * QN + (1.0 - epsi) * F_QN[gi]);
          F_NN[gi] = (epsi * NN + (1.0 - epsi) * F_NN[gi]);
          F_QN[gi] = fmax32((double)f1em24, F_QN[gi]);
          double cs4d = F_QN[gi] / F_NN[gi];
          cs4d = fmax32((double)f1em24, cs4d);
          // :390-421
          double beta = (bexp == 1.0) ? cs4d / cs2d : std::pow(cs4d / cs2d, bexp);
          if (jz == nz) beta = 1.0;
          Beta[gi] = beta;
          double betaclip = fmax32(beta, 1.0 / (tf1 * tf2));
          double cs = cs2d / betaclip;
          Cs_opt2[gi] = fmax32((double)f1em24, cs);
          sum2d += cs2d; sumcs += Cs_opt2[gi]; sum4d += cs4d;
        }
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = nx + 1; jx <= ld; ++jx) Cs_opt2[o + (size_t)(jx - 1) + (size_t)ld * (jy - 1)] = (double)f1em24;
      Beta_avg[jz - 1] = sum2d / sumcs;
      Betaclip_avg[jz - 1] = sum4d / sum2d;
    }
  }

  // lagrange_scalar_Sdep.f90:1-467 (model 7; inilag = .false., inflow =
  // .false., lbc = 1): Cs2_Pr = Cs^2 / Pr_t from Lagrangian averages of the
  // scalar's L.M and Q.N along the pathlines, relaxed with the time scales
  // lagrange_Sdep left in TnLMMM, TnQNNN; Pr_t = Cs_opt2 / Cs2_Pr; Beta is
  // overwritten with the scalar's scale-dependence factor.
  void lagrange_scalar_Sdep(double* cs2_pr, const double* s11, const double* s12, const double* s13,
                            const double* s22, const double* s23, const double* s33) {
    const double delta = 1.0 * std::pow(dx * dy, 1.0 / 2.0);  // :61
    const double tf1 = 2.0, tf2 = 4.0;
    const double opftdelta = 1.5 * delta;  // opftime = 1.5
    const Field u_temp = u, v_temp = v, theta_temp = theta;  // :72-74
    interpolag_scalar_Sdep();  // :76
    const double lagran_dt = dt * (double)cs_count;  // :79
    const double cst = delta * delta;  // const = delta**2 (:81)
    // :83-87: theta is Nyquist-filtered in place; the derivatives are local
    Field ldTdx(nfield, 0.0), ldTdy(nfield, 0.0), ldTdz(nfield, 0.0);
    filt_da(theta.data(), ldTdx.data(), ldTdy.data(), nz);
    ddz_uv(ldTdz.data(), theta.data());
    for (size_t i = 0; i < nplane; ++i) ldTdz[(size_t)(nz - 1) * nplane + i] = dTdz_top / T_scale * z_i;
    {  // :96-131, lbc = 1: the mean surface flux and the mean u*
      double slz = 0.0, sws = 0.0, sus = 0.0, spm = 0.0;
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= nx; ++jx) slz += std::log(zo[S2(jx, jy)]);
      const double zo_avg = std::exp(slz / (double)(float)(nx * ny));
      for (size_t q = 0; q < wt_s.size(); ++q) sws += wt_s[q];
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= nx; ++jx) {
          const size_t i = I(jx, jy, 1);
          sus += std::sqrt(u[i] * u[i] + v[i] * v[i]);
          spm += psi_m[S2(jx, jy)];
        }
      const double ustar_ = sus / (double)(float)(nx * ny) * vonk /
                            (std::log(0.5 * dz / zo_avg) - spm / (double)(float)(nx * ny));
      const double sflux = (sws / (double)(nx * ny)) / T_scale / u_star;
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= nx; ++jx)
          ldTdz[I(jx, jy, 1)] = -phi_h[S2(jx, jy)] * sflux / (ustar_ * vonk * dz / 2.0);
    }
    const float f1em24 = 1e-24f;
    const double bexp = std::log(tf1) / (std::log(tf2) - std::log(tf1));
#pragma omp parallel for schedule(static)
    for (int jz = 1; jz <= nz; ++jz) {
      const size_t NP = nplane, o = (size_t)(jz - 1) * NP;
      // planes: 0..3 u,v,w,theta bar ; 4..7 hat ; 8..10 L ; 11..13 Q ; 14..19 S bar ;
      // 20..25 S hat ; 26..28 S dT bar ; 29..31 S dT hat ; 32..34 dT bar ; 35..37 dT hat
      std::vector<double> buf(NP * 38);
      auto pl = [&](int q) { return buf.data() + (size_t)q * NP; };
      for (size_t i = 0; i < NP; ++i) {
        double ub, vb, wb, tb;
        if (jz == 1) {  // :140-145
          ub = u_temp[i]; vb = v_temp[i]; wb = 0.25 * w[NP + i]; tb = theta_temp[i];
        } else {
          ub = 0.5 * (u_temp[o + i] + u_temp[o - NP + i]);
          vb = 0.5 * (v_temp[o + i] + v_temp[o - NP + i]);
          wb = w[o + i];
          tb = 0.5 * (theta_temp[o + i] + theta_temp[o - NP + i]);
        }
        pl(0)[i] = ub; pl(1)[i] = vb; pl(2)[i] = wb; pl(3)[i] = tb;
        pl(4)[i] = ub; pl(5)[i] = vb; pl(6)[i] = wb; pl(7)[i] = tb;
        pl(8)[i] = ub * tb; pl(9)[i] = vb * tb; pl(10)[i] = wb * tb;
        pl(11)[i] = ub * tb; pl(12)[i] = vb * tb; pl(13)[i] = wb * tb;
      }
      for (int q = 0; q < 4; ++q) test_filter(pl(q), G_test);  // :166-169
      for (int q = 0; q < 3; ++q) {  // :171-176
        test_filter(pl(8 + q), G_test);
        for (size_t i = 0; i < NP; ++i) pl(8 + q)[i] = pl(8 + q)[i] - pl(q)[i] * pl(3)[i];
      }
      for (int q = 0; q < 4; ++q) test_filter(pl(4 + q), G_test_test);  // :178-181
      for (int q = 0; q < 3; ++q) {  // :183-188
        test_filter(pl(11 + q), G_test_test);
        for (size_t i = 0; i < NP; ++i) pl(11 + q)[i] = pl(11 + q)[i] - pl(4 + q)[i] * pl(7)[i];
      }
      const double* Sp[6] = {s11 + o, s12 + o, s13 + o, s22 + o, s23 + o, s33 + o};
      std::vector<double> S(NP);
      for (size_t i = 0; i < NP; ++i) {
        S[i] = smag(Sp[0][i], Sp[3][i], Sp[5][i], Sp[1][i], Sp[2][i], Sp[4][i]);  // :190-191
        for (int q = 0; q < 6; ++q) { pl(14 + q)[i] = Sp[q][i]; pl(20 + q)[i] = Sp[q][i]; }
        double dx_, dy_, dz_;
        if (jz == 1) {  // :227-235
          dx_ = ldTdx[o + i]; dy_ = ldTdy[o + i]; dz_ = (ldTdz[o + i] + ldTdz[o + NP + i]) / 2.0;
          pl(26)[i] = S[i] * ldTdx[o + i];
          pl(27)[i] = S[i] * ldTdy[o + i];
          pl(28)[i] = S[i] * (ldTdz[o + i] + ldTdz[o + NP + i]) / 2.0;
        } else {
          dx_ = (ldTdx[o + i] + ldTdx[o - NP + i]) / 2.0;
          dy_ = (ldTdy[o + i] + ldTdy[o - NP + i]) / 2.0;
          dz_ = ldTdz[o + i];
          pl(26)[i] = S[i] * (ldTdx[o + i] + ldTdx[o - NP + i]) / 2.0;
          pl(27)[i] = S[i] * (ldTdy[o + i] + ldTdy[o - NP + i]) / 2.0;
          pl(28)[i] = S[i] * ldTdz[o + i];
        }
        pl(29)[i] = pl(26)[i]; pl(30)[i] = pl(27)[i]; pl(31)[i] = pl(28)[i];
        pl(32)[i] = dx_; pl(33)[i] = dy_; pl(34)[i] = dz_;  // :253-262
        pl(35)[i] = dx_; pl(36)[i] = dy_; pl(37)[i] = dz_;
      }
      for (int q = 0; q < 6; ++q) test_filter(pl(14 + q), G_test);  // :208-220
      for (int q = 0; q < 6; ++q) test_filter(pl(20 + q), G_test_test);
      for (int q = 0; q < 3; ++q) test_filter(pl(26 + q), G_test);  // :241-247
      for (int q = 0; q < 3; ++q) test_filter(pl(29 + q), G_test_test);
      for (int q = 0; q < 3; ++q) test_filter(pl(32 + q), G_test);  // :268-274
      for (int q = 0; q < 3; ++q) test_filter(pl(35 + q), G_test_test);
      // columns 1:nx; the padding columns (Cs2_Pr = Cs_opt2 = 1e-24 there,
      // :334-336, :384-386) carry Pr_t = 1 and feed nothing back
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = nx + 1; jx <= ld; ++jx) {
          Pr_t[o + (size_t)(jx - 1) + (size_t)ld * (jy - 1)] = 1.0;
          cs2_pr[o + (size_t)(jx - 1) + (size_t)ld * (jy - 1)] = (double)f1em24;
        }
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= nx; ++jx) {
          const size_t i = (size_t)(jx - 1) + (size_t)ld * (jy - 1);
          const size_t gi = o + i;
          const double Sb = smag(pl(14)[i], pl(17)[i], pl(19)[i], pl(15)[i], pl(16)[i], pl(18)[i]);
          const double Sh = smag(pl(20)[i], pl(23)[i], pl(25)[i], pl(21)[i], pl(22)[i], pl(24)[i]);
          double M[3], N[3];
          for (int q = 0; q < 3; ++q) {  // :276-282
            M[q] = cst * (pl(26 + q)[i] - 4.0 * Sb * pl(32 + q)[i]);
            N[q] = cst * (pl(29 + q)[i] - 16.0 * Sh * pl(35 + q)[i]);
          }
          const double LM = pl(8)[i] * M[0] + pl(9)[i] * M[1] + pl(10)[i] * M[2];  // :286-289
          const double MM = M[0] * M[0] + M[1] * M[1] + M[2] * M[2];
          const double QN = pl(11)[i] * N[0] + pl(12)[i] * N[1] + pl(13)[i] * N[2];
          const double NN = N[0] * N[0] + N[1] * N[1] + N[2] * N[2];
          // :322-332
          double Tn = opftdelta * pow_m18(TnLMMM[gi]);
          Tn = fmax32((double)f1em24, Tn);
          double dumfac = lagran_dt / Tn;
          double epsi = dumfac / (1.0 + dumfac);
          G_LM[gi] = (epsi * LM + (1.0 - epsi) * G_LM[gi]);
          G_MM[gi] = (epsi * MM + (1.0 - epsi) * G_MM[gi]);
          G_LM[gi] = fmax32((double)f1em24, G_LM[gi]);
          double c2 = G_LM[gi] / G_MM[gi];  // :334-337
          c2 = fmax32((double)f1em24, c2);
          // :350-365
          Tn = opftdelta * pow_m18(TnQNNN[gi]);
          Tn = fmax32((double)f1em24, Tn);
          dumfac = lagran_dt / Tn;
          epsi = dumfac / (1.0 + dumfac);
          G_QN[gi] = (epsi * QN + (1.0 - epsi) * G_QN[gi]);
          G_NN[gi] = (epsi * NN + (1.0 - epsi) * G_NN[gi]);
          G_QN[gi] = fmax32((double)f1em24, G_QN[gi]);
          double c4 = G_QN[gi] / G_NN[gi];
          c4 = fmax32((double)f1em24, c4);
          // :367-388
          double beta = (bexp == 1.0) ? c4 / c2 : std::pow(c4 / c2, bexp);
          if (jz == nz) beta = 1.0;
          Beta[gi] = beta;
          const double betaclip = fmax32(beta, 1.0 / (tf1 * tf2));
          double cp = c2 / betaclip;
          cp = fmax32((double)f1em24, cp);
          cs2_pr[gi] = cp;
          Pr_t[gi] = Cs_opt2[gi] / cp;  // :390
        }
    }
  }

  // sgsmodule.f90:37-59
  static double rtnewt(const double* A) {
    double x1 = 0.0, x2 = 15.0, xacc = 0.001;
    double r = 0.5 * (x1 + x2);
    for (int j = 1; j <= 100; ++j) {
      double f = A[0] + r * (A[1] + r * (A[2] + r * (A[3] + r * (A[4] + r * A[5]))));
      double df = A[1] + r * (2.0 * A[2] + r * (3.0 * A[3] + r * (4.0 * A[4] + r * (5.0 * A[5]))));
      double d = f / df;
      r = r - d;
      if (std::fabs(d) < xacc) return r;
    }
    return 1.0;
  }

  // std_dynamic.f90:1-136 (model 2): per level, u, v, w on w-nodes and their
  // products (:33-61), G_test (2 delta) filtered, L_ij = (uu)~ - u~u~
  // (:64-78); S_ij and |S| S_ij filtered (:83-117); M_ij = 2 delta^2
  // (|S|S_ij~ - 4 |S~| S_ij~) (:120-127) with delta = filter_size
  // (dx dy dz)^(1/3) (:28, unlike the (dx dy)^(1/2) of sgs_stag and
  // scaledep_dynamic); Cs^2(jz) = max(0, sum L_ij M_ij / sum M_ij M_ij)
  // (:130-133).  The sums
  // run over 1:nx: the (ld,ny) sums of the reference add the two padding
  // columns, which hold zero after the test filter (G_test's kx = nx/2
  // column is zero).
  void std_dynamic(double* cs_z, const double* s11, const double* s12, const double* s13, const double* s22,
                   const double* s23, const double* s33) {
    const double delta = 1.0 * std::pow(dx * dy * dz, 1.0 / 3.0);
#pragma omp parallel for schedule(static)
    for (int jz = 1; jz <= nz; ++jz) {
      const size_t NP = nplane, o = (size_t)(jz - 1) * NP;
      std::vector<double> buf(NP * 21);
      auto pl = [&](int q) { return buf.data() + (size_t)q * NP; };
      for (size_t i = 0; i < NP; ++i) {  // :33-61
        double ub, vb, wb;
        if (jz == 1) {
          ub = u[i]; vb = v[i]; wb = 0.25 * w[NP + i];
          pl(3)[i] = u[i] * u[i]; pl(4)[i] = u[i] * v[i]; pl(5)[i] = u[i] * 0.25 * w[NP + i];
          pl(6)[i] = v[i] * v[i]; pl(7)[i] = v[i] * 0.25 * w[NP + i];
          const double t = 0.25 * w[NP + i];
          pl(8)[i] = t * t;
        } else {
          ub = 0.5 * (u[o + i] + u[o - NP + i]);
          vb = 0.5 * (v[o + i] + v[o - NP + i]);
          wb = w[o + i];
          pl(3)[i] = 0.5 * (u[o + i] + u[o - NP + i]) * 0.5 * (u[o + i] + u[o - NP + i]);
          pl(4)[i] = 0.5 * (u[o + i] + u[o - NP + i]) * 0.5 * (v[o + i] + v[o - NP + i]);
          pl(5)[i] = 0.5 * (u[o + i] + u[o - NP + i]) * w[o + i];
          pl(6)[i] = 0.5 * (v[o + i] + v[o - NP + i]) * 0.5 * (v[o + i] + v[o - NP + i]);
          pl(7)[i] = 0.5 * (v[o + i] + v[o - NP + i]) * w[o + i];
          pl(8)[i] = w[o + i] * w[o + i];
        }
        pl(0)[i] = ub; pl(1)[i] = vb; pl(2)[i] = wb;
      }
      const int ia[6] = {0, 0, 0, 1, 1, 2}, ib[6] = {0, 1, 2, 1, 2, 2};
      for (int q = 0; q < 3; ++q) test_filter(pl(q), G_test);
      for (int q = 0; q < 6; ++q) {  // :64-78
        test_filter(pl(3 + q), G_test);
        for (size_t i = 0; i < NP; ++i) pl(3 + q)[i] = pl(3 + q)[i] - pl(ia[q])[i] * pl(ib[q])[i];
      }
      const double* Sp[6] = {s11 + o, s12 + o, s13 + o, s22 + o, s23 + o, s33 + o};
      for (size_t i = 0; i < NP; ++i) {  // :83-111
        const double S = smag(Sp[0][i], Sp[3][i], Sp[5][i], Sp[1][i], Sp[2][i], Sp[4][i]);
        for (int q = 0; q < 6; ++q) { pl(9 + q)[i] = Sp[q][i]; pl(15 + q)[i] = S * Sp[q][i]; }
      }
      for (int q = 0; q < 12; ++q) test_filter(pl(9 + q), G_test);
      const double cst = 2.0 * (delta * delta);
      double num = 0.0, den = 0.0;
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= nx; ++jx) {
          const size_t i = (size_t)(jx - 1) + (size_t)ld * (jy - 1);
          double b[6], sb[6], Lq[6], M[6];
          for (int q = 0; q < 6; ++q) { b[q] = pl(9 + q)[i]; sb[q] = pl(15 + q)[i]; Lq[q] = pl(3 + q)[i]; }
          const double Sb = smag(b[0], b[3], b[5], b[1], b[2], b[4]);  // :102-103
          for (int q = 0; q < 6; ++q) M[q] = cst * (sb[q] - 4.0 * Sb * b[q]);
          num += Lq[0] * M[0] + Lq[3] * M[3] + Lq[5] * M[5] + 2.0 * (Lq[1] * M[1] + Lq[2] * M[2] + Lq[4] * M[4]);
          den += M[0] * M[0] + M[3] * M[3] + M[5] * M[5] + 2.0 * (M[1] * M[1] + M[2] * M[2] + M[4] * M[4]);
        }
      cs_z[jz - 1] = std::max(0.0, num / den);
    }
  }

  // scaledep_dynamic.f90:4-255 (sums over 1:nx)
  void scaledep_dynamic(double* cs_z, const double* s11, const double* s12, const double* s13,
                        const double* s22, const double* s23, const double* s33) {
    const double delta = 1.0 * std::pow(dx * dy, 1.0 / 2.0);
    const double N2 = (double)(nx * ny);
#pragma omp parallel for schedule(static)
    for (int jz = 1; jz <= nz; ++jz) {
      const size_t NP = nplane, o = (size_t)(jz - 1) * NP;
      std::vector<double> buf(NP * 42);
      auto pl = [&](int q) { return buf.data() + (size_t)q * NP; };
      for (size_t i = 0; i < NP; ++i) {
        double ub, vb, wb;
        if (jz == 1) {
          ub = u[i]; vb = v[i]; wb = 0.25 * w[NP + i];
          pl(6)[i] = u[i] * u[i]; pl(7)[i] = u[i] * v[i]; pl(8)[i] = u[i] * 0.25 * w[NP + i];
          pl(9)[i] = v[i] * v[i]; pl(10)[i] = v[i] * 0.25 * w[NP + i];
          double t = 0.25 * w[NP + i]; pl(11)[i] = t * t;
        } else {
          ub = 0.5 * (u[o + i] + u[o - NP + i]);
          vb = 0.5 * (v[o + i] + v[o - NP + i]);
          wb = w[o + i];
          pl(6)[i] = 0.5 * (u[o + i] + u[o - NP + i]) * 0.5 * (u[o + i] + u[o - NP + i]);
          pl(7)[i] = 0.5 * (u[o + i] + u[o - NP + i]) * 0.5 * (v[o + i] + v[o - NP + i]);
          pl(8)[i] = 0.5 * (u[o + i] + u[o - NP + i]) * w[o + i];
          pl(9)[i] = 0.5 * (v[o + i] + v[o - NP + i]) * 0.5 * (v[o + i] + v[o - NP + i]);
          pl(10)[i] = 0.5 * (v[o + i] + v[o - NP + i]) * w[o + i];
          pl(11)[i] = w[o + i] * w[o + i];
        }
        pl(0)[i] = ub; pl(1)[i] = vb; pl(2)[i] = wb;
        pl(3)[i] = ub; pl(4)[i] = vb; pl(5)[i] = wb;
      }
      const int ia[6] = {0, 0, 0, 1, 1, 2}, ib[6] = {0, 1, 2, 1, 2, 2};
      for (int q = 0; q < 3; ++q) test_filter(pl(q), G_test);
      for (int q = 0; q < 6; ++q) {
        test_filter(pl(6 + q), G_test);
        for (size_t i = 0; i < NP; ++i) pl(6 + q)[i] = pl(6 + q)[i] - pl(ia[q])[i] * pl(ib[q])[i];
      }
      for (int q = 0; q < 6; ++q)
        for (size_t i = 0; i < NP; ++i) pl(12 + q)[i] = pl(ia[q])[i] * pl(ib[q])[i];
      for (int q = 0; q < 3; ++q) test_filter(pl(3 + q), G_test_test);
      for (int q = 0; q < 6; ++q) {
        test_filter(pl(12 + q), G_test_test);
        for (size_t i = 0; i < NP; ++i) pl(12 + q)[i] = pl(12 + q)[i] - pl(3 + ia[q])[i] * pl(3 + ib[q])[i];
      }
      const double* Sp[6] = {s11 + o, s12 + o, s13 + o, s22 + o, s23 + o, s33 + o};
      std::vector<double> S(NP);
      for (size_t i = 0; i < NP; ++i) {
        S[i] = smag(Sp[0][i], Sp[3][i], Sp[5][i], Sp[1][i], Sp[2][i], Sp[4][i]);
        for (int q = 0; q < 6; ++q) {
          pl(18 + q)[i] = Sp[q][i]; pl(24 + q)[i] = Sp[q][i];
          pl(30 + q)[i] = S[i] * Sp[q][i]; pl(36 + q)[i] = S[i] * Sp[q][i];
        }
      }
      for (int q = 0; q < 6; ++q) test_filter(pl(18 + q), G_test);
      for (int q = 0; q < 6; ++q) test_filter(pl(24 + q), G_test_test);
      for (int q = 0; q < 6; ++q) test_filter(pl(30 + q), G_test);
      for (int q = 0; q < 6; ++q) test_filter(pl(36 + q), G_test_test);
      double sa1 = 0, sb1 = 0, sc1 = 0, sd1 = 0, se1 = 0, sa2 = 0, sb2 = 0, sc2 = 0, sd2 = 0, se2 = 0;
      std::vector<double> Sbar(NP), Shat(NP);
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= nx; ++jx) {
          const size_t i = (size_t)(jx - 1) + (size_t)ld * (jy - 1);
          const double *L = nullptr; (void)L;
          double b[6], h[6], Sb_[6], Sh_[6], Lq[6], Qq[6];
          for (int q = 0; q < 6; ++q) {
            b[q] = pl(18 + q)[i]; h[q] = pl(24 + q)[i]; Sb_[q] = pl(30 + q)[i]; Sh_[q] = pl(36 + q)[i];
            Lq[q] = pl(6 + q)[i]; Qq[q] = pl(12 + q)[i];
          }
          const double Sb = smag(b[0], b[3], b[5], b[1], b[2], b[4]);
          const double Sh = smag(h[0], h[3], h[5], h[1], h[2], h[4]);
          Sbar[i] = Sb; Shat[i] = Sh;
          sa1 += Sb * (b[0] * Lq[0] + b[3] * Lq[3] + b[5] * Lq[5] + 2.0 * (b[1] * Lq[1] + b[2] * Lq[2] + b[4] * Lq[4]));
          sb1 += Sb_[0] * Lq[0] + Sb_[3] * Lq[3] + Sb_[5] * Lq[5] + 2.0 * (Sb_[1] * Lq[1] + Sb_[2] * Lq[2] + Sb_[4] * Lq[4]);
          sc1 += Sb_[0] * Sb_[0] + Sb_[3] * Sb_[3] + Sb_[5] * Sb_[5] + 2.0 * (Sb_[1] * Sb_[1] + Sb_[2] * Sb_[2] + Sb_[4] * Sb_[4]);
          sd1 += 0.5 * (Sb * Sb * Sb * Sb);
          se1 += Sb * (b[0] * Sb_[0] + b[3] * Sb_[3] + b[5] * Sb_[5] + 2.0 * (b[1] * Sb_[1] + b[2] * Sb_[2] + b[4] * Sb_[4]));
          sa2 += Sh * (h[0] * Qq[0] + h[3] * Qq[3] + h[5] * Qq[5] + 2.0 * (h[1] * Qq[1] + h[2] * Qq[2] + h[4] * Qq[4]));
          sb2 += Sh_[0] * Qq[0] + Sh_[3] * Qq[3] + Sh_[5] * Qq[5] + 2.0 * (Sh_[1] * Qq[1] + Sh_[2] * Qq[2] + Sh_[4] * Qq[4]);
          sc2 += Sh_[0] * Sh_[0] + Sh_[3] * Sh_[3] + Sh_[5] * Sh_[5] + 2.0 * (Sh_[1] * Sh_[1] + Sh_[2] * Sh_[2] + Sh_[4] * Sh_[4]);
          sd2 += 0.5 * (Sh * Sh * Sh * Sh);
          se2 += Sh * (h[0] * Sh_[0] + h[3] * Sh_[3] + h[5] * Sh_[5] + 2.0 * (h[1] * Sh_[1] + h[2] * Sh_[2] + h[4] * Sh_[4]));
        }
      const double d2 = delta * delta;
      const double t2 = (2.0 * d2) * (2.0 * d2);
      const double a1 = -2.0 * d2 * 4.0 * sa1 / N2;
      const double b1 = -2.0 * d2 * sb1 / N2;
      const double c1 = t2 * sc1 / N2;
      const double d1 = t2 * 16.0 * sd1 / N2;
      const double e1 = 2.0 * t2 * 4.0 * se1 / N2;
      const double a2 = -2.0 * d2 * 16.0 * sa2 / N2;
      const double b2 = -2.0 * d2 * sb2 / N2;
      const double c2 = t2 * sc2 / N2;
      const double d2_ = t2 * 256.0 * sd2 / N2;
      const double e2 = 2.0 * t2 * 16.0 * se2 / N2;
      double A[6];
      A[0] = b2 * c1 - b1 * c2;
      A[1] = a1 * c2 - b2 * e1;
      A[2] = b2 * d1 + b1 * e2 - a2 * c1;
      A[3] = a2 * e1 - a1 * e2;
      A[4] = -a2 * d1 - b1 * d2_;
      A[5] = a1 * d2_;
      const double beta = rtnewt(A);
      const double cst = 2.0 * d2;
      double num = 0.0, den = 0.0;
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= nx; ++jx) {
          const size_t i = (size_t)(jx - 1) + (size_t)ld * (jy - 1);
          double M[6];
          for (int q = 0; q < 6; ++q) M[q] = cst * (pl(30 + q)[i] - 4.0 * beta * Sbar[i] * pl(18 + q)[i]);
          double Lq[6];
          for (int q = 0; q < 6; ++q) Lq[q] = pl(6 + q)[i];
          num += Lq[0] * M[0] + Lq[3] * M[3] + Lq[5] * M[5] + 2.0 * (Lq[1] * M[1] + Lq[2] * M[2] + Lq[4] * M[4]);
          den += M[0] * M[0] + M[3] * M[3] + M[5] * M[5] + 2.0 * (M[1] * M[1] + M[2] * M[2] + M[4] * M[4]);
        }
      double cz = num / den;
      cs_z[jz - 1] = std::max(0.0, cz);
    }
  }

  // wallstress.f90:5-69 ('wall', WALL_HOMOG_FLAG = .false.)
  void wallstress() {
    std::vector<double> u1(nplane), v1(nplane);
    for (size_t i = 0; i < nplane; ++i) { u1[i] = u[i]; v1[i] = v[i]; }
    test_filter(u1.data(), G_test_test);
    test_filter(v1.data(), G_test_test);
    for (int jy = 1; jy <= ny; ++jy)
      for (int jx = 1; jx <= nx; ++jx) {
        const size_t s = S2(jx, jy), i = I(jx, jy, 1);
        const double denom = std::log(0.5 * dz / zo[s]) - psi_m[s] + psi_m0[s];
        const double u_avg = std::sqrt(u1[i] * u1[i] + v1[i] * v1[i]);
        ustar_avg[s] = u_avg * vonk / denom;
        const double cst = -(ustar_avg[s] * ustar_avg[s]) / u_avg;
        txz[i] = cst * u1[i];
        tyz[i] = cst * v1[i];
        double a = ustar_avg[s] / (0.5 * dz * vonk) * u1[i] / u_avg * phi_m[s];
        double b = ustar_avg[s] / (0.5 * dz * vonk) * v1[i] / u_avg * phi_m[s];
        dudz[i] = (u[i] == 0.0) ? 0.0 : a;
        dvdz[i] = (v[i] == 0.0) ? 0.0 : b;
      }
  }

  // scalars_module.f90:508-690 (patch_flag = 1)
  void obukhov() {
    if (jt == 1) {  // SCAL_init = 1
      std::fill(psi_m.begin(), psi_m.end(), 0.0);
      std::fill(psi_m0.begin(), psi_m0.end(), 0.0);
      std::fill(psi_h.begin(), psi_h.end(), 0.0);
      std::fill(psi_h0.begin(), psi_h0.end(), 0.0);
      if (!initsc) {
        for (size_t s = 0; s < sgs_t3.size(); ++s) sgs_t3[s] = wt_s[s] / (u_star * T_scale);
        if (q_flag)
          for (size_t s = 0; s < sgs_q3.size(); ++s) sgs_q3[s] = wq_s[s] / (u_star * q_scale);
      }
    }
    const double g_ = (g * z_i) / (u_star * u_star);
    double th = 0.0;
    for (int jy = 1; jy <= ny; ++jy)
      for (int jx = 1; jx <= nx; ++jx) th += theta[I(jx, jy, 1)];
    const double theta_ = th / (double)(float)(nx * ny);
    std::vector<double> u1(nplane), v1(nplane);
    for (size_t i = 0; i < nplane; ++i) { u1[i] = u[i]; v1[i] = v[i]; }
    test_filter(u1.data(), G_test_test);
    test_filter(v1.data(), G_test_test);
    for (int jx = 1; jx <= nx; ++jx)
      for (int jy = 1; jy <= ny; ++jy) {
        const size_t s = S2(jx, jy), i = I(jx, jy, 1);
        const double u_avg = std::sqrt(u1[i] * u1[i] + v1[i] * v1[i]);
        ustar_avg[s] = u_avg * vonk / (std::log(0.5 * dz / zo[s]) - psi_m[s] + psi_m0[s]);
      }
    for (int jx = 1; jx <= nx; ++jx)
      for (int jy = 1; jy <= ny; ++jy) {
        const size_t s = S2(jx, jy);
        const double wt_avg = sgs_t3[s];
        const double wtv_avg = q_flag ? sgs_t3[s] + 0.61 * theta[I(jx, jy, 1)] * (0.001 * q_scale * sgs_q3[s])
                                      : sgs_t3[s] + 0.61 * theta[I(jx, jy, 1)] * (0.001 * 100.0 * 0.0);
        const double us = ustar_avg[s];
        const double L = -(us * us * us) / (vonk * (g_ / theta_) * wtv_avg);
        double zeta = 0.5 * dz / L, zeta0 = zo[s] / L, zeta0s = z_os[s] / L;
        if (zeta < -30.0) zeta = -30.0;
        if (zeta > 2.0) zeta = 2.0;
        if (zeta0 < -30.0) zeta0 = -30.0;
        if (zeta0 > 2.0) zeta0 = 2.0;
        if (zeta0s < -30.0) zeta0s = -30.0;
        if (zeta0s > 2.0) zeta0s = 2.0;
        if (L < 0.0 && wt_avg != 0.0) {
          const double x = std::pow(1.0 - 16.0 * zeta, 0.25);
          psi_m[s] = 2.0 * std::log((1.0 + x) / 2.0) + std::log((1.0 + x * x) / 2.0) - 2.0 * std::atan(x) + PI / 2.0;
          psi_h[s] = 2.0 * std::log((1.0 + x * x) / 2.0);
          phi_m[s] = 1.0 / x;
          phi_h[s] = 1.0 / (x * x);
          const double x0 = std::pow(1.0 - 16.0 * zeta0, 0.25);
          const double x0s = std::pow(1.0 - 16.0 * zeta0s, 0.25);
          psi_m0[s] = 2.0 * std::log((1.0 + x0) / 2.0) + std::log((1.0 + x0 * x0) / 2.0) - 2.0 * std::atan(x0) + PI / 2.0;
          psi_h0[s] = 2.0 * std::log((1.0 + x0s * x0s) / 2.0);
        } else if (L > 0.0 && wt_avg != 0.0) {
          phi_m[s] = 1.0 + 5.0 * zeta;
          phi_h[s] = 1.0 + 5.0 * zeta;
          psi_m[s] = -1.0 * 5.0 * zeta;
          psi_h[s] = -1.0 * 5.0 * zeta;
          psi_m0[s] = -1.0 * 5.0 * zeta0;
          psi_h0[s] = -1.0 * 5.0 * zeta0s;
        } else {
          psi_m[s] = 0.0; psi_m0[s] = 0.0; psi_h[s] = 0.0; psi_h0[s] = 0.0;
          phi_m[s] = 1.0; phi_h[s] = 1.0;
        }
      }
  }

  // divstress_uv.f90:1-63
  void divstress_uv(double* divt, const double* tx, const double* ty, const double* tz) {
    std::vector<double> dtxdx(nfield), dtydy(nfield), dtzdz(nfield, 0.0);
    ddx(dtxdx.data(), tx, nz);
    ddy(dtydy.data(), ty, nz);
    ddz_w(dtzdz.data(), tz);
    for (size_t i = 0; i < nplane * (nz - 1); ++i) divt[i] = dtxdx[i] + dtydy[i] + dtzdz[i];
    for (int jz = 1; jz <= nz - 1; ++jz)
      for (int jy = 1; jy <= ny; ++jy) { divt[I(ld - 1, jy, jz)] = 0.0; divt[I(ld, jy, jz)] = 0.0; }
    for (size_t i = 0; i < nplane; ++i) divt[(size_t)(nz - 1) * nplane + i] = BOGUS;
  }
  // divstress_w.f90:4-86
  void divstress_w(double* divt, const double* tx, const double* ty, const double* tz) {
    std::vector<double> dtxdx(nfield), dtydy(nfield), dtzdz(nfield, 0.0);
    ddx(dtxdx.data(), tx, nz);
    ddy(dtydy.data(), ty, nz);
    ddz_uv(dtzdz.data(), tz);
    for (int jy = 1; jy <= ny; ++jy)
      for (int jx = 1; jx <= nx; ++jx) { const size_t i = I(jx, jy, 1); divt[i] = dtxdx[i] + dtydy[i]; }
    for (int jz = 2; jz <= nz - 1; ++jz)
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= nx; ++jx) { const size_t i = I(jx, jy, jz); divt[i] = dtxdx[i] + dtydy[i] + dtzdz[i]; }
    for (int jz = 1; jz <= nz - 1; ++jz)
      for (int jy = 1; jy <= ny; ++jy) { divt[I(ld - 1, jy, jz)] = 0.0; divt[I(ld, jy, jz)] = 0.0; }
    for (int jy = 1; jy <= ny; ++jy)
      for (int jx = 1; jx <= nx; ++jx) { const size_t i = I(jx, jy, nz); divt[i] = dtxdx[i] + dtydy[i] + dtzdz[i]; }
    for (int jy = 1; jy <= ny; ++jy) { divt[I(ld - 1, jy, nz)] = 0.0; divt[I(ld, jy, nz)] = 0.0; }
  }

  // tridag_array.f90:1-109 ; a,b,c real (lh,ny,n), r,uu complex (lh,ny,n), n = nz+1
  int tridag_array(const double* a, const double* b, const double* c, const double* r, double* uu) {
    const int n = nz + 1;
    const size_t NK = (size_t)lh * ny;
    auto R = [&](const double* x, int jx, int jy, int j) { return &x[2 * ((size_t)(jx - 1) + (size_t)lh * (jy - 1) + NK * (j - 1))]; };
    auto Rr = [&](const double* x, int jx, int jy, int j) { return x[(size_t)(jx - 1) + (size_t)lh * (jy - 1) + NK * (j - 1)]; };
    for (int jy = 1; jy <= ny; ++jy)
      for (int jx = 1; jx <= lh - 1; ++jx)
        if (Rr(b, jx, jy, 1) == 0.0) return LES_ERR_PIVOT;
    std::vector<double> bet(NK), gam(NK * n);
    for (int jy = 1; jy <= ny; ++jy)
      for (int jx = 1; jx <= lh; ++jx) {
        const size_t k = (size_t)(jx - 1) + (size_t)lh * (jy - 1);
        bet[k] = Rr(b, jx, jy, 1);
        const double* rr = R(r, jx, jy, 1);
        double* o = const_cast<double*>(R(uu, jx, jy, 1));
        o[0] = rr[0] / bet[k];
        o[1] = rr[1] / bet[k];
      }
    int status = LES_OK;
    for (int j = 2; j <= n; ++j)
      for (int jy = 1; jy <= ny; ++jy) {
        if (jy == ny / 2 + 1) continue;
        for (int jx = 1; jx <= lh - 1; ++jx) {
          if (jx * jy == 1) continue;
          const size_t k = (size_t)(jx - 1) + (size_t)lh * (jy - 1);
          gam[k + NK * (j - 1)] = Rr(c, jx, jy, j - 1) / bet[k];
          bet[k] = Rr(b, jx, jy, j) - Rr(a, jx, jy, j) * gam[k + NK * (j - 1)];
          if (bet[k] == 0.0) status = LES_ERR_PIVOT;
          const double* rr = R(r, jx, jy, j);
          const double* up = R(uu, jx, jy, j - 1);
          double* o = const_cast<double*>(R(uu, jx, jy, j));
          const double aa = Rr(a, jx, jy, j);
          o[0] = (rr[0] - aa * up[0]) / bet[k];
          o[1] = (rr[1] - aa * up[1]) / bet[k];
        }
      }
    for (int j = n - 1; j >= 1; --j)
      for (int jy = 1; jy <= ny; ++jy) {
        if (jy == ny / 2 + 1) continue;
        for (int jx = 1; jx <= lh - 1; ++jx) {
          if (jx * jy == 1) continue;
          const size_t k = (size_t)(jx - 1) + (size_t)lh * (jy - 1);
          double* o = const_cast<double*>(R(uu, jx, jy, j));
          const double* up = R(uu, jx, jy, j + 1);
          const double gg = gam[k + NK * j];
          o[0] = o[0] - gg * up[0];
          o[1] = o[1] - gg * up[1];
        }
      }
    return status;
  }

  // press_stag_array.f90:1-294 ; p_hat (ld,ny,0:nz), dfdx/dfdy (ld,ny,nz)
  int press_stag_array(double* p_hat, double* dfdx, double* dfdy) {
    const size_t NP = nplane;
    for (size_t i = 0; i < NP; ++i) p_hat[i] = 0.0;  // p_hat(:,:,0) = 0
    const double cst = 1.0 / (double)(nx * ny);
    std::vector<double> rHx(nfield, 0.0), rHy(nfield, 0.0), rHz(nfield, 0.0);
#pragma omp parallel for schedule(static)
    for (int jz = 1; jz <= nz - 1; ++jz) {
      const size_t o = (size_t)(jz - 1) * NP;
      for (size_t i = 0; i < NP; ++i) {
        rHx[o + i] = cst / TADV1 * (u[o + i] / dt);
        rHy[o + i] = cst / TADV1 * (v[o + i] / dt);
        rHz[o + i] = cst / TADV1 * (w[o + i] / dt);
      }
      fs->r2c(&rHx[o]); fs->r2c(&rHy[o]); fs->r2c(&rHz[o]);
    }
    {
      const size_t o = (size_t)(nz - 1) * NP;
      for (size_t i = 0; i < NP; ++i) { rHx[o + i] = BOGUS; rHy[o + i] = BOGUS; rHz[o + i] = 0.0; }
    }
    std::vector<double> rbot(NP), rtop(NP);
    for (size_t i = 0; i < NP; ++i) {
      rbot[i] = cst * divtz[i];
      rtop[i] = cst * divtz[(size_t)(nz - 1) * NP + i];
    }
    fs->r2c(rbot.data());
    fs->r2c(rtop.data());
    for (int jz = 1; jz <= nz - 1; ++jz) {
      kill_oddballs(&rHx[(size_t)(jz - 1) * NP]);
      kill_oddballs(&rHy[(size_t)(jz - 1) * NP]);
      kill_oddballs(&rHz[(size_t)(jz - 1) * NP]);
    }
    kill_oddballs(rtop.data());
    kill_oddballs(rbot.data());
    const int n = nz + 1;
    const size_t NK = (size_t)lh * ny;
    std::vector<double> a(NK * n, 0.0), b(NK * n, 0.0), c(NK * n, 0.0), rc(2 * NK * n, 0.0), uc(2 * NK * n, 0.0);
    auto Kk = [&](int jx, int jy) { return (size_t)(jx - 1) + (size_t)lh * (jy - 1); };
    for (int jy = 1; jy <= ny; ++jy)
      for (int jx = 1; jx <= lh; ++jx) {
        const size_t k = Kk(jx, jy);
        a[k] = BOGUS; b[k] = -1.0; c[k] = 1.0;
        rc[2 * k] = -dz * RE(rbot.data(), ld, jx, jy);
        rc[2 * k + 1] = -dz * IM(rbot.data(), ld, jx, jy);
        const size_t kt = k + NK * (size_t)(n - 1);
        a[kt] = -1.0; b[kt] = 1.0; c[kt] = BOGUS;
        rc[2 * kt] = -RE(rtop.data(), ld, jx, jy) * dz;
        rc[2 * kt + 1] = -IM(rtop.data(), ld, jx, jy) * dz;
      }
    const double idz2 = 1.0 / (dz * dz);
    for (int jz = 2; jz <= nz; ++jz)
      for (int jy = 1; jy <= ny; ++jy) {
        if (jy == ny / 2 + 1) continue;
        for (int jx = 1; jx <= lh - 1; ++jx) {
          if (jx * jy == 1) continue;
          const size_t k = Kk(jx, jy) + NK * (size_t)(jz - 1);
          const double kxx = kx[Kk(jx, jy)], kyy = ky[Kk(jx, jy)];
          a[k] = idz2;
          b[k] = -(kxx * kxx + kyy * kyy + 2.0 / (dz * dz));
          c[k] = idz2;
          double* Hx = &rHx[(size_t)(jz - 2) * NP];
          double* Hy = &rHy[(size_t)(jz - 2) * NP];
          double* Hz0 = &rHz[(size_t)(jz - 2) * NP];
          double* Hz1 = &rHz[(size_t)(jz - 1) * NP];
          const double sr = kxx * RE(Hx, ld, jx, jy) + kyy * RE(Hy, ld, jx, jy);
          const double si = kxx * IM(Hx, ld, jx, jy) + kyy * IM(Hy, ld, jx, jy);
          rc[2 * k] = -si + (RE(Hz1, ld, jx, jy) - RE(Hz0, ld, jx, jy)) / dz;
          rc[2 * k + 1] = sr + (IM(Hz1, ld, jx, jy) - IM(Hz0, ld, jx, jy)) / dz;
        }
      }
    int st = tridag_array(a.data(), b.data(), c.data(), rc.data(), uc.data());
    // u(:,:,j) -> p_hat(:,:,j-1) (complex view)
    for (int jz = 0; jz <= nz; ++jz)
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= lh; ++jx) {
          const size_t k = Kk(jx, jy) + NK * (size_t)jz;
          double* pl = p_hat + (size_t)jz * NP;
          RE(pl, ld, jx, jy) = uc[2 * k];
          IM(pl, ld, jx, jy) = uc[2 * k + 1];
        }
    // zero-wavenumber mode :238-247
    RE(p_hat, ld, 1, 1) = 0.0; IM(p_hat, ld, 1, 1) = 0.0;
    {
      double* p1 = p_hat + NP;
      RE(p1, ld, 1, 1) = RE(p_hat, ld, 1, 1) - dz * RE(rbot.data(), ld, 1, 1);
      IM(p1, ld, 1, 1) = IM(p_hat, ld, 1, 1) - dz * IM(rbot.data(), ld, 1, 1);
    }
    for (int jz = 2; jz <= nz; ++jz) {
      double* pc = p_hat + (size_t)jz * NP;
      double* pp = p_hat + (size_t)(jz - 1) * NP;
      double* Hz = &rHz[(size_t)(jz - 1) * NP];
      RE(pc, ld, 1, 1) = RE(pp, ld, 1, 1) + RE(Hz, ld, 1, 1) * dz;
      IM(pc, ld, 1, 1) = IM(pp, ld, 1, 1) + IM(Hz, ld, 1, 1) * dz;
    }
    for (int jz = 0; jz <= nz; ++jz) kill_oddballs(p_hat + (size_t)jz * NP);
    fs->c2r(p_hat);
#pragma omp parallel for schedule(static)
    for (int jz = 1; jz <= nz - 1; ++jz) {
      double* pl = p_hat + (size_t)jz * NP;
      double* xp = dfdx + (size_t)(jz - 1) * NP;
      double* yp = dfdy + (size_t)(jz - 1) * NP;
      eye_k(xp, pl, kx);
      eye_k(yp, pl, ky);
      fs->c2r(xp);
      fs->c2r(yp);
      fs->c2r(pl);
    }
    for (size_t i = 0; i < NP; ++i) {
      dfdx[(size_t)(nz - 1) * NP + i] = BOGUS;
      dfdy[(size_t)(nz - 1) * NP + i] = BOGUS;
      p_hat[(size_t)nz * NP + i] = BOGUS;
    }
    return st;
  }

  // forcing.f90:128-219 (fx = fy = fz = 0, inflow = .false.)
  void project() {
    for (int jz = 1; jz <= nz - 1; ++jz)
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= nx; ++jx) {
          const size_t i = I(jx, jy, jz);
          double RHS = -TADV1 * dpdx[i];
          u[i] = (u[i] + dt * (RHS + 0.0));
          RHS = -TADV1 * dpdy[i];
          v[i] = (v[i] + dt * (RHS + 0.0));
        }
    for (int jz = 2; jz <= nz - 1; ++jz)
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= nx; ++jx) {
          const size_t i = I(jx, jy, jz);
          double RHS = -TADV1 * dpdz[i];
          w[i] = (w[i] + dt * (RHS + 0.0));
        }
    const size_t ot = (size_t)(nz - 1) * nplane, ob = (size_t)(nz - 2) * nplane;
    for (size_t i = 0; i < nplane; ++i) {
      u[ot + i] = u[ob + i];
      v[ot + i] = v[ob + i];
      w[ot + i] = 0.0;
      w[i] = 0.0;
    }
  }

  // scalars_module.f90:232-454 scalar_RHS_calc (theta) and
  // scalars_module_q.f90:145-367 scalar_q_RHS_calc (qmix): the same
  // algorithm on the scalar's arrays; the surface flux is wt_s/(T_scale u_star)
  // for theta and wq_s/q_scale/u_star for qmix (lbc = 1)
  void scalar_RHS_calc(const Field& scalar, Field& dsdx, Field& dsdy, Field& dsdz, Field& RHS, const Field& flux,
                       Field& sgs_vert, Field& sgs_vol, bool humidity) {
    std::vector<double> ustar_local = ustar_avg;
    std::vector<double> sn1(nplane);
    for (size_t i = 0; i < nplane; ++i) sn1[i] = scalar[i];
    test_filter(sn1.data(), G_test);
    std::vector<double> surf_flux((size_t)nx * ny, 0.0);
    if (scalar[0] < 2.0) {  // lbc == 1
      for (int i = 1; i <= nx; ++i)
        for (int j = 1; j <= ny; ++j)
          surf_flux[S2(i, j)] = humidity ? flux[S2(i, j)] / q_scale / u_star : flux[S2(i, j)] / (T_scale * u_star);
    }
    for (int i = 1; i <= nx; ++i)
      for (int j = 1; j <= ny; ++j) {
        const size_t s = S2(i, j);
        dsdz[I(i, j, 1)] = -phi_h[s] * surf_flux[s] / (ustar_local[s] * vonk * dz / 2.0);
      }
    const size_t NB = nplane_big * nz;
    std::vector<double> u_m(NB), v_m(NB), w_m(NB), dsdx_m(NB), dsdy_m(NB), dsdz_m(NB), RHS_m(NB, 0.0);
    dealias1(u.data(), u_m.data(), nz);
    dealias1(v.data(), v_m.data(), nz);
    dealias1(w.data(), w_m.data(), nz);
    dealias1(dsdx.data(), dsdx_m.data(), nz);
    dealias1(dsdy.data(), dsdy_m.data(), nz);
    dealias1(dsdz.data(), dsdz_m.data(), nz);
    auto Bi = [&](int i, int j, int k) { return (size_t)(i - 1) + (size_t)ld_big * ((size_t)(j - 1) + (size_t)ny2 * (k - 1)); };
    for (int k = 2; k <= nz - 1; ++k)
      for (int j = 1; j <= ny2; ++j)
        for (int i = 1; i <= nx2; ++i) {
          const size_t a = Bi(i, j, k), b = Bi(i, j, k + 1);
          RHS_m[a] = u_m[a] * dsdx_m[a] + v_m[a] * dsdy_m[a] + (w_m[a] * dsdz_m[a] + w_m[b] * dsdz_m[b]) / 2.0;
        }
    for (int j = 1; j <= ny2; ++j)
      for (int i = 1; i <= nx2; ++i) {
        const size_t a = Bi(i, j, 1), b = Bi(i, j, 2);
        RHS_m[a] = u_m[a] * dsdx_m[a] + v_m[a] * dsdy_m[a] + (0.5 * w_m[b]) * dsdz_m[b];
      }
    for (int j = 1; j <= ny2; ++j)
      for (int i = 1; i <= nx2; ++i) {
        const size_t a = Bi(i, j, nz);
        RHS_m[a] = u_m[a] * dsdx_m[a] + v_m[a] * dsdy_m[a];
      }
    dealias2(RHS.data(), RHS_m.data(), nz);
    std::vector<double> temp(nfield, 0.0), dtemp(nfield, 0.0);
    // Pr_ (scalars_module.f90:77-82): Pr for models 1-5, the field Pr_t otherwise
    auto Pr_ = [&](size_t a) { return model == 7 ? Pr_t[a] : Pr; };
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        const size_t a = I(i, j, 1);
        temp[a] = (1.0 / Pr_(a)) * Nu_t[a] * dsdx[a];
      }
    for (int k = 2; k <= nz - 1; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          const size_t a = I(i, j, k), b = I(i, j, k + 1);
          temp[a] = (1.0 / (0.5 * (Pr_(a) + Pr_(b)))) * 0.5 * (Nu_t[a] + Nu_t[b]) * dsdx[a];
        }
    ddx(dtemp.data(), temp.data(), nz);
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        const size_t a = I(i, j, 1);
        RHS[a] = (-1.0 * RHS[a] + dtemp[a]);
        temp[a] = (1.0 / Pr_(a)) * Nu_t[a] * dsdy[a];
      }
    for (int k = 2; k <= nz - 1; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          const size_t a = I(i, j, k), b = I(i, j, k + 1);
          RHS[a] = (-1.0 * RHS[a] + dtemp[a]);
          temp[a] = (1.0 / (0.5 * (Pr_(a) + Pr_(b)))) * 0.5 * (Nu_t[a] + Nu_t[b]) * dsdy[a];
        }
    ddy(dtemp.data(), temp.data(), nz);
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        const size_t a = I(i, j, 1);
        RHS[a] = RHS[a] + dtemp[a];
        temp[a] = -1.0 * surf_flux[S2(i, j)];
        sgs_vert[S2(i, j)] = surf_flux[S2(i, j)];
        sgs_vol[a] = surf_flux[S2(i, j)];
      }
    for (int k = 2; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          const size_t a = I(i, j, k);
          RHS[a] = RHS[a] + dtemp[a];
          temp[a] = (1.0 / Pr_(a)) * Nu_t[a] * dsdz[a];
          sgs_vol[a] = -1.0 * temp[a];
        }
    std::fill(dtemp.begin(), dtemp.end(), 0.0);
    ddz_w(dtemp.data(), temp.data());
    for (int k = 1; k <= nz - 1; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          const size_t a = I(i, j, k);
          RHS[a] = RHS[a] + dtemp[a];
        }
  }

  // scalars_module.f90:175-228 calcbeta(theta, qmix): the virtual
  // temperature theta (1 + 0.61 * 0.001 qmix q_scale) (qmix = 0 without humidity)
  void calcbeta() {
    const double g_hat = g * (z_i / (u_star * u_star));
    std::fill(beta_scal.begin(), beta_scal.end(), 0.0);
    auto tv = [&](size_t a) {
      return q_flag ? theta[a] * (1 + 0.61 * 0.001 * qmix[a] * q_scale) : theta[a] * 1.0;
    };
    std::vector<double> sb(nz + 1, 0.0);
    for (int k = 1; k <= nz; ++k) {
      double s = 0.0;
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i)
          s = s + (q_flag ? tv(I(i, j, k)) : theta[I(i, j, k)] * (1.0 + 0.61 * 0.001 * 0.0 * 100.0));
      sb[k] = s / (double)(nx * ny);
    }
    for (int k = 2; k <= nz - 1; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          const double above = (tv(I(i, j, k)) - sb[k]) / sb[k];
          const double below = (tv(I(i, j, k - 1)) - sb[k - 1]) / sb[k - 1];
          beta_scal[I(i, j, k)] = g_hat * (above + below) / 2.0;
        }
  }

  // scalars_module.f90:457-504 step_scalar / scalars_module_q.f90:370-397
  // step_scalar_q; the lid value follows the gradient when L_z > z_i
  // (a one-process domain: L_z nproc = L_z), else it copies level nz-1
  void step_scalar(Field& scalar, const Field& RHS, const Field& RHSf, double top_grad) {
    for (int k = 1; k <= nz - 1; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          const size_t a = I(i, j, k);
          scalar[a] = scalar[a] + dt * (1.5 * RHS[a] - 0.5 * RHSf[a]);
        }
    const size_t ot = (size_t)(nz - 1) * nplane, ob = (size_t)(nz - 2) * nplane;
    if (cfg.lz_over_zi > 1.0) {
      const double inc = top_grad * dz;
      for (size_t i = 0; i < nplane; ++i) scalar[ot + i] = scalar[ob + i] + inc;
    } else {
      for (size_t i = 0; i < nplane; ++i) scalar[ot + i] = scalar[ob + i];
    }
  }

  // scalars_module.f90:57-171
  void theta_all_in_one() {
    filt_da(theta.data(), dTdx.data(), dTdy.data(), nz);
    ddz_uv(dTdz.data(), theta.data());
    {
      const double top = dTdz_top / T_scale * z_i;
      for (size_t i = 0; i < nplane; ++i) dTdz[(size_t)(nz - 1) * nplane + i] = top;
    }
    RHS_Tf = RHS_T;
    scalar_RHS_calc(theta, dTdx, dTdy, dTdz, RHS_T, wt_s, sgs_t3, sgs_t3_vol, false);
    calcbeta();
    if (jt == 1 && !initsc) RHS_Tf = RHS_T;
    step_scalar(theta, RHS_T, RHS_Tf, dTdz_top / T_scale * z_i);
  }

  // scalars_module_q.f90:31-141 (Pr_ = Pr for models 1-5)
  void q_all_in_one() {
    filt_da(qmix.data(), dqdx.data(), dqdy.data(), nz);
    ddz_uv(dqdz.data(), qmix.data());
    {
      const double top = dqdz_top / q_scale * z_i;
      for (size_t i = 0; i < nplane; ++i) dqdz[(size_t)(nz - 1) * nplane + i] = top;
    }
    RHS_qf = RHS_q;
    scalar_RHS_calc(qmix, dqdx, dqdy, dqdz, RHS_q, wq_s, sgs_q3, sgs_q3_vol, true);
    if (jt == 1 && !initsc) RHS_qf = RHS_q;
    step_scalar(qmix, RHS_q, RHS_qf, dqdz_top / q_scale * z_i);
  }

  // atm_thermodynamics.f90:37-52 (k_global = jz), columns 1..nx; out: actual_T,
  // actual_Tv, sat_vapor_pr, pr_atm, vapor_pr, sat_qmix, rel_hum, rel_hum_q, zlcl_all
  void thermo(double* const* out) {
    const double cp = 1005.0, Rd = 287.04, pr_surf = 100000.0;  // param.f90:90-96
    for (int k = 0; k < 9; ++k) std::fill(out[k], out[k] + nfield, 0.0);
    for (int jz = 1; jz <= nz - 1; ++jz)
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= nx; ++jx) {
          const size_t a = I(jx, jy, jz);
          const double zg = jz * dz * z_i;
          const double aT = theta[a] - (g / cp) * (zg) / T_scale;
          const double aTv = aT * (1 + 0.61 * 0.001 * qmix[a] * q_scale);
          const double svp = 611.2 * std::exp(17.62 * (aT * T_scale - 273.2) / (243.12 + (aT * T_scale - 273.2)));
          const double pa = pr_surf * std::exp(-(zg) / (Rd * aTv * T_scale / g));
          const double vp = (0.001 * q_scale * qmix[a] / (0.001 * q_scale * qmix[a] + 0.622)) * pa;
          const double sq = 0.622 * svp / (pa - svp);
          const double rh = vp / svp;
          const double rhq = 0.001 * q_scale * qmix[a] / sq;
          const double zl = zg + (cp / g) * (aT * T_scale - 55 - std::pow(1 / (aT * T_scale - 55) - std::log(rhq) / 2840, -1.0));
          out[0][a] = aT; out[1][a] = aTv; out[2][a] = svp; out[3][a] = pa; out[4][a] = vp;
          out[5][a] = sq; out[6][a] = rh; out[7][a] = rhq; out[8][a] = zl;
        }
  }

  // io.f90:403-1218 MM_XYZ_Out, the accumulation (the output files are the
  // caller's): statistics by the reference's array names
  Field& st(const char* name) {
    for (size_t i = 0; i < stat_names.size(); ++i)
      if (stat_names[i] == name) return stats[i];
    stat_names.push_back(name);
    stats.emplace_back((size_t)nx * ny * (nz - 1), 0.0);
    return stats.back();
  }
  void stats_enable(int c_count, int p_count) {
    stats_c = c_count;
    stats_p = p_count;
    for (Field& f : stats) std::fill(f.begin(), f.end(), 0.0);
  }
  void stats_accumulate() {
    const size_t SN = (size_t)nx * ny * (nz - 1);
    static const char* const all[] = {
        "au", "av", "aw", "ap", "atheta", "aq", "p2", "u2", "v2", "w2", "theta2", "q2", "u3", "v3", "w3", "q3",
        "T3", "adudx", "adudy", "adudz", "advdx", "advdy", "advdz", "adwdx", "adwdy", "adwdz", "adTdx", "adTdy",
        "adTdz", "adqdx", "adqdy", "adqdz", "adpdx", "adpdy", "adpdz", "tke", "awe", "aue", "ave", "auw", "avw",
        "awt", "awq", "aut", "avt", "auq", "avq", "auv", "awuu", "awvv", "awqq", "awtt", "awwu", "awwv", "awwt",
        "awwq", "atxx", "atxz", "atyy", "atyz", "atzz", "aup", "avp", "awp", "atp", "aqp", "atq", "aupx", "aupy",
        "aupz", "avpx", "avpy", "avpz", "awpx", "awpy", "awpz", "at11ux", "at12uy", "at13uz", "at21vx", "at22vy",
        "at23vz", "at31wx", "at32wy", "at33wz", "apux", "apuy", "apuz", "apvx", "apvy", "apvz", "apwx", "apwy",
        "apwz", "aptx", "apty", "aptz", "apqx", "apqy", "apqz", "at11s11", "at12s12", "at13s13", "at22s22",
        "at23s23", "at33s33", "as11", "as12", "as13", "as22", "as23", "as33", "aut11", "aut12", "aut13", "avt21",
        "avt22", "avt23", "awt31", "awt32", "awt33", "asgst3", "asgsq3", "aactual_T", "aactual_Tv", "apr_atm",
        "arel_hum", "arel_hum_q", "avapor_pr", "asat_vapor_pr", "asat_qmix", "azlcl_all"};
    for (const char* nm : all) st(nm);
    st("atxy");  // never zeroed (io.f90:457-502 and the output blocks leave it out)
    if (jt_total <= stats_c)  // io.f90:457
      for (const char* nm : all) std::fill(st(nm).begin(), st(nm).end(), 0.0);
    // atm_thermodynamics.f90:37-52 of the current theta, qmix (thermo() ran
    // on them at the end of the step)
    std::vector<Field> th(9, Field(nfield, 0.0));
    {
      const double cp = 1005.0, Rd = 287.04, pr_surf = 100000.0;
      for (int jz = 1; jz <= nz - 1; ++jz)
        for (int jy = 1; jy <= ny; ++jy)
          for (int jx = 1; jx <= nx; ++jx) {
            const size_t a = I(jx, jy, jz);
            const double qa = q_flag ? qmix[a] : 0.0;
            const double zg = jz * dz * z_i;
            const double aT = theta[a] - (g / cp) * (zg) / T_scale;
            const double aTv = aT * (1 + 0.61 * 0.001 * qa * q_scale);
            const double svp = 611.2 * std::exp(17.62 * (aT * T_scale - 273.2) / (243.12 + (aT * T_scale - 273.2)));
            const double pa = pr_surf * std::exp(-(zg) / (Rd * aTv * T_scale / g));
            const double vp = (0.001 * q_scale * qa / (0.001 * q_scale * qa + 0.622)) * pa;
            const double sq = 0.622 * svp / (pa - svp);
            const double rhq = 0.001 * q_scale * qa / sq;
            th[0][a] = aT; th[1][a] = aTv; th[2][a] = svp; th[3][a] = pa; th[4][a] = vp; th[5][a] = sq;
            th[6][a] = vp / svp; th[7][a] = rhq;
            th[8][a] = zg + (cp / g) * (aT * T_scale - 55 - std::pow(1 / (aT * T_scale - 55) - std::log(rhq) / 2840, -1.0));
          }
    }
    const double fr = (1.0 / (double)stats_p) * (double)stats_c;  // io.f90:504
    auto Q = [&](const Field& f, size_t a) { return q_flag ? f[a] : 0.0; };
    std::map<std::string, double*> ptr;
    for (size_t i = 0; i < stat_names.size(); ++i) ptr[stat_names[i]] = stats[i].data();
    for (int k = 1; k <= nz - 1; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          const size_t a = I(i, j, k), o = (size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (k - 1));
          double arg1, arg2, arg3, arg4, arg7, arg8, ux, uy, uz, vx, vy, vz, wx, wy, wz, px, py, pz, tx, ty, tz, qx,
              qy, qz;
          if (k == 1) {  // io.f90:531-581
            const size_t b = I(i, j, k + 1);
            arg1 = u[a]; arg2 = v[a]; arg3 = 0.25 * w[b];
            arg4 = p[P(i, j, k)] - 0.5 * (arg1 * arg1 + arg2 * arg2 + arg3 * arg3);
            arg7 = theta[a]; arg8 = Q(qmix, a);
            ux = dudx[a]; uy = dudy[a]; uz = dudz[a];
            vx = dvdx[a]; vy = dvdy[a]; vz = dvdz[a];
            wx = ((dwdx[b]) / 2.0); wy = ((dwdy[b]) / 2.0); wz = dwdz[a];
            px = dpdx[a] - arg1 * ux - arg2 * vx - arg3 * wx;
            py = dpdy[a] - arg1 * uy - arg2 * vy - arg3 * wy;
            pz = dpdz[a] - arg1 * uz - arg2 * vz - arg3 * wz;
            tx = dTdx[a]; ty = dTdy[a]; tz = dTdz[a];
            qx = Q(dqdx, a); qy = Q(dqdy, a); qz = Q(dqdz, a);
          } else {  // io.f90:583-622
            const size_t m = I(i, j, k - 1);
            arg1 = (u[a] + u[m]) / 2.0; arg2 = (v[a] + v[m]) / 2.0; arg3 = w[a];
            arg4 = ((p[P(i, j, k)] + p[P(i, j, k - 1)]) / 2.0 - 0.5 * (arg1 * arg1 + arg2 * arg2 + arg3 * arg3));
            arg7 = (theta[a] + theta[m]) / 2.0; arg8 = (Q(qmix, a) + Q(qmix, m)) / 2.0;
            ux = ((dudx[a] + dudx[m]) / 2.0); uy = ((dudy[a] + dudy[m]) / 2.0); uz = dudz[a];
            vx = ((dvdx[a] + dvdx[m]) / 2.0); vy = ((dvdy[a] + dvdy[m]) / 2.0); vz = dvdz[a];
            wx = dwdx[a]; wy = dwdy[a]; wz = ((dwdz[a] + dwdz[m]) / 2.0);
            px = ((dpdx[a] + dpdx[m]) / 2.0) - arg1 * ux - arg2 * vx - arg3 * wx;
            py = ((dpdy[a] + dpdy[m]) / 2.0) - arg1 * uy - arg2 * vy - arg3 * wy;
            pz = dpdz[a] - arg1 * uz - arg2 * vz - arg3 * wz;
            tx = ((dTdx[a] + dTdx[m]) / 2.0); ty = ((dTdy[a] + dTdy[m]) / 2.0); tz = dTdz[a];
            qx = ((Q(dqdx, a) + Q(dqdx, m)) / 2.0); qy = ((Q(dqdy, a) + Q(dqdy, m)) / 2.0); qz = Q(dqdz, a);
          }
          auto A = [&](const char* nm, double val) { double* f = ptr.at(nm); f[o] = f[o] + val; };
          // io.f90:628-639
          A("aactual_T", fr * th[0][a] * T_scale); A("aactual_Tv", fr * th[1][a] * T_scale);
          A("apr_atm", fr * th[3][a]); A("arel_hum", fr * th[6][a]); A("arel_hum_q", fr * th[7][a]);
          A("avapor_pr", fr * th[4][a]); A("asat_vapor_pr", fr * th[2][a]); A("asat_qmix", fr * th[5][a]);
          A("azlcl_all", fr * th[8][a]);
          // io.f90:642-717
          A("au", fr * arg1); A("av", fr * arg2); A("aw", fr * arg3); A("ap", fr * arg4);
          A("atheta", fr * arg7); A("aq", fr * arg8);
          A("u2", fr * arg1 * arg1); A("v2", fr * arg2 * arg2); A("w2", fr * arg3 * arg3);
          A("p2", fr * arg4 * arg4); A("theta2", fr * arg7 * arg7); A("q2", fr * arg8 * arg8);
          A("tke", fr * (0.5 * (arg1 * arg1 + arg2 * arg2 + arg3 * arg3)));
          A("u3", fr * arg1 * arg1 * arg1); A("v3", fr * arg2 * arg2 * arg2); A("w3", fr * arg3 * arg3 * arg3);
          A("T3", fr * arg7 * arg7 * arg7); A("q3", fr * arg8 * arg8 * arg8);
          A("awe", fr * arg3 * (0.5 * (arg1 * arg1 + arg2 * arg2 + arg3 * arg3)));
          A("ave", fr * arg2 * (0.5 * (arg1 * arg1 + arg2 * arg2 + arg3 * arg3)));
          A("aue", fr * arg1 * (0.5 * (arg1 * arg1 + arg2 * arg2 + arg3 * arg3)));
          A("auw", fr * arg1 * arg3); A("avw", fr * arg2 * arg3); A("awt", fr * arg3 * arg7);
          A("awq", fr * arg3 * arg8); A("auv", fr * arg1 * arg2); A("aut", fr * arg1 * arg7);
          A("avt", fr * arg2 * arg7); A("auq", fr * arg1 * arg8); A("avq", fr * arg2 * arg8);
          A("awuu", fr * arg3 * arg1 * arg1); A("awvv", fr * arg3 * arg2 * arg2); A("awtt", fr * arg3 * arg7 * arg7);
          A("awqq", fr * arg3 * arg8 * arg8); A("awwu", fr * arg3 * arg3 * arg1); A("awwv", fr * arg3 * arg3 * arg2);
          A("awwt", fr * arg3 * arg3 * arg7); A("awwq", fr * arg3 * arg3 * arg8);
          A("asgst3", fr * (sgs_t3_vol[a]));
          A("asgsq3", fr * (q_flag ? sgs_q3_vol[a] : 0.0));
          // io.f90:751-773
          A("adudx", fr * ux); A("adudy", fr * uy); A("adudz", fr * uz);
          A("advdx", fr * vx); A("advdy", fr * vy); A("advdz", fr * vz);
          A("adwdx", fr * wx); A("adwdy", fr * wy); A("adwdz", fr * wz);
          A("adTdx", fr * tx); A("adTdy", fr * ty); A("adTdz", fr * tz);
          A("adqdx", fr * qx); A("adqdy", fr * qy); A("adqdz", fr * qz);
          A("adpdx", fr * px); A("adpdy", fr * py); A("adpdz", fr * pz);
          // io.f90:778-846
          A("atxx", fr * txx[a]); A("atxy", fr * txy[a]); A("atxz", fr * txz[a]);
          A("atyz", fr * tyz[a]); A("atyy", fr * tyy[a]); A("atzz", fr * tzz[a]);
          A("aup", fr * arg1 * arg4); A("avp", fr * arg2 * arg4); A("awp", fr * arg3 * arg4);
          A("atp", fr * arg7 * arg4); A("aqp", fr * arg8 * arg4); A("atq", fr * arg7 * arg8);
          A("aupx", fr * arg1 * px); A("aupy", fr * arg1 * py); A("aupz", fr * arg1 * pz);
          A("avpx", fr * arg2 * px); A("avpy", fr * arg2 * py); A("avpz", fr * arg2 * pz);
          A("awpx", fr * arg3 * px); A("awpy", fr * arg3 * py); A("awpz", fr * arg3 * pz);
          A("at11ux", fr * txx[a] * dudx[a]); A("at12uy", fr * txy[a] * dudy[a]); A("at13uz", fr * txz[a] * dudz[a]);
          A("at21vx", fr * txy[a] * dvdx[a]); A("at22vy", fr * tyy[a] * dvdy[a]); A("at23vz", fr * tyz[a] * dvdz[a]);
          A("at31wx", fr * txz[a] * dwdx[a]); A("at32wy", fr * tyz[a] * dwdy[a]); A("at33wz", fr * tzz[a] * dwdz[a]);
          A("apux", fr * arg4 * ux); A("apuy", fr * arg4 * uy); A("apuz", fr * arg4 * uz);
          A("apvx", fr * arg4 * vx); A("apvy", fr * arg4 * vy); A("apvz", fr * arg4 * vz);
          A("apwx", fr * arg4 * wx); A("apwy", fr * arg4 * wy); A("apwz", fr * arg4 * wz);
          A("aptx", fr * arg4 * tx); A("apty", fr * arg4 * ty); A("aptz", fr * arg4 * tz);
          A("apqx", fr * arg4 * qx); A("apqy", fr * arg4 * qy); A("apqz", fr * arg4 * qz);
          // io.f90:851-876
          const double S11_ = ux, S12_ = 0.5 * (uy + vx), S13_ = 0.5 * (uz + wx);
          const double S22_ = vy, S23_ = 0.5 * (vz + wy), S33_ = wz;
          A("as11", fr * S11_); A("as12", fr * S12_); A("as13", fr * S13_);
          A("as22", fr * S22_); A("as23", fr * S23_); A("as33", fr * S33_);
          A("at11s11", fr * txx[a] * S11_); A("at12s12", fr * txy[a] * S12_); A("at13s13", fr * txz[a] * S13_);
          A("at22s22", fr * tyy[a] * S22_); A("at23s23", fr * tyz[a] * S23_); A("at33s33", fr * tzz[a] * S33_);
          A("aut11", fr * txx[a] * arg1); A("aut12", fr * txy[a] * arg1); A("aut13", fr * txz[a] * arg1);
          A("avt21", fr * txy[a] * arg2); A("avt22", fr * tyy[a] * arg2); A("avt23", fr * tyz[a] * arg2);
          A("awt31", fr * txz[a] * arg3); A("awt32", fr * tyz[a] * arg3); A("awt33", fr * tzz[a] * arg3);
        }
    (void)SN;
  }
  // the zeroing after output, io.f90:997-1006 (group 1, every p_count steps)
  // and io.f90:1189-1216 (group 2, every 2 p_count steps)
  void stats_reset(int group) {
    static const char* const g1[] = {"au", "av", "aw", "atheta", "aq", "u2", "v2", "w2", "theta2", "q2", "auw",
                                     "avw", "awt", "awq", "atxz", "atyz", "asgst3", "asgsq3", "azlcl_all"};
    static const char* const g2[] = {
        "ap", "p2", "u3", "v3", "w3", "q3", "T3", "adudx", "adudy", "adudz", "advdx", "advdy", "advdz", "adwdx",
        "adwdy", "adwdz", "adTdx", "adTdy", "adTdz", "adqdx", "adqdy", "adqdz", "adpdx", "adpdy", "adpdz", "tke",
        "awe", "aue", "ave", "aut", "avt", "auq", "avq", "auv", "awuu", "awvv", "awqq", "awtt", "awwu", "awwv",
        "awwt", "awwq", "atxx", "atyy", "atzz", "aup", "avp", "awp", "atp", "aqp", "atq", "aupx", "aupy", "aupz",
        "avpx", "avpy", "avpz", "awpx", "awpy", "awpz", "at11ux", "at12uy", "at13uz", "at21vx", "at22vy", "at23vz",
        "at31wx", "at32wy", "at33wz", "apux", "apuy", "apuz", "apvx", "apvy", "apvz", "apwx", "apwy", "apwz",
        "aptx", "apty", "aptz", "apqx", "apqy", "apqz", "at11s11", "at12s12", "at13s13", "at22s22", "at23s23",
        "at33s33", "as11", "as12", "as13", "as22", "as23", "as33", "aut11", "aut12", "aut13", "avt21", "avt22",
        "avt23", "awt31", "awt32", "awt33", "aactual_T", "aactual_Tv", "apr_atm", "arel_hum", "arel_hum_q",
        "avapor_pr", "asat_vapor_pr", "asat_qmix"};
    if (group == 1)
      for (const char* nm : g1) std::fill(st(nm).begin(), st(nm).end(), 0.0);
    if (group == 2)
      for (const char* nm : g2) std::fill(st(nm).begin(), st(nm).end(), 0.0);
  }

  // rmsdiv.f90:1-113
  double rmsdiv() {
    double rms = 0.0;
    for (int jz = 1; jz <= nz - 1; ++jz)
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= nx; ++jx) {
          const size_t i = I(jx, jy, jz);
          rms = rms + std::fabs(dudx[i] + dvdy[i] + dwdz[i]);
        }
    return rms / (double)(nx * ny * (nz - 1));
  }
  // scalars_module2.f90:22-70 (non-MPI)
  void timestep_conditions(double* cflu, double* visc) {
    double umax = -1e300, numax = -1e300;
    for (int jz = 1; jz <= nz - 1; ++jz)
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= nx; ++jx) {
          const size_t i = I(jx, jy, jz);
          umax = std::max(umax, u[i] * u[i] + v[i] * v[i] + w[i] * w[i]);
          numax = std::max(numax, Nu_t[i]);
        }
    const double u_res_max = std::sqrt(umax);
    const double delta = std::min(dx, dy);
    *cflu = u_res_max * dt / dx;
    *visc = dt * numax / (delta * delta);
  }

  // main.f90:202-478, one iteration
  int step() {
    jt += 1;
    jt_total += 1;
    tt = tt + dt;
    RHSx_f = RHSx; RHSy_f = RHSy; RHSz_f = RHSz;
    obukhov();
    filt_da(u.data(), dudx.data(), dudy.data(), nz);
    filt_da(v.data(), dvdx.data(), dvdy.data(), nz);
    filt_da(w.data(), dwdx.data(), dwdy.data(), nz);
    ddz_uv(dudz.data(), u.data());
    ddz_uv(dvdz.data(), v.data());
    ddz_w(dwdz.data(), w.data());
    wallstress();
    sgs_stag();
    if (s_flag) {  // main.f90:272-275 (thermo writes diagnostics only)
      theta_all_in_one();
      if (q_flag) q_all_in_one();
    } else {
      std::fill(beta_scal.begin(), beta_scal.end(), 0.0);
    }
    divstress_uv(divtx.data(), txx.data(), txy.data(), txz.data());
    divstress_uv(divty.data(), txy.data(), tyy.data(), tyz.data());
    divstress_w(divtz.data(), txz.data(), tyz.data(), tzz.data());
    convec(RHSx.data(), RHSy.data(), RHSz.data());
    const size_t nv = nplane * (nz - 1);
    for (size_t i = 0; i < nv; ++i) {
      RHSx[i] = -RHSx[i] - divtx[i];
      RHSy[i] = -RHSy[i] - divty[i];
      RHSz[i] = -RHSz[i] - divtz[i];
    }
    if (s_flag)
      for (size_t i = 0; i < nv; ++i) RHSz[i] = RHSz[i] + beta_scal[i];
    if (jt == 1 && !initu) { RHSx_f = RHSx; RHSy_f = RHSy; RHSz_f = RHSz; }
    for (size_t i = 0; i < nv; ++i) {
      u[i] = u[i] + dt * (TADV1 * RHSx[i] + TADV2 * RHSx_f[i] + 0.0);
      v[i] = v[i] + dt * (TADV1 * RHSy[i] + TADV2 * RHSy_f[i]);
      w[i] = w[i] + dt * (TADV1 * RHSz[i] + TADV2 * RHSz_f[i]);
    }
    for (size_t i = 0; i < nplane; ++i) {
      const size_t o = (size_t)(nz - 1) * nplane + i;
      u[o] = BOGUS; v[o] = BOGUS; w[o] = BOGUS;
    }
    int st = press_stag_array(p.data(), dpdx.data(), dpdy.data());
    for (int jz = 1; jz <= nz - 1; ++jz)
      for (int jy = 1; jy <= ny; ++jy)
        for (int jx = 1; jx <= nx; ++jx)
          dpdz[I(jx, jy, jz)] = (p[P(jx, jy, jz)] - p[P(jx, jy, jz - 1)]) / dz;
    for (size_t i = 0; i < nplane; ++i) dpdz[(size_t)(nz - 1) * nplane + i] = BOGUS;
    for (size_t i = 0; i < nv; ++i) {
      RHSx[i] = RHSx[i] - dpdx[i];
      RHSy[i] = RHSy[i] - dpdy[i];
      RHSz[i] = RHSz[i] - dpdz[i];
    }
    project();
    if (cfg.rmsdiv_every > 0 && jt % cfg.rmsdiv_every == 0) {
      rmsdiv_last = rmsdiv();
      double cflu, visc;
      timestep_conditions(&cflu, &visc);
      if (cflu > 0.1 || cflu < 0.0) return LES_ERR_CFL;
    }
    return st;
  }

  Field* field(int id) {
    switch (id) {
      case LES_U: return &u; case LES_V: return &v; case LES_W: return &w; case LES_THETA: return &theta;
      case LES_DUDX: return &dudx; case LES_DUDY: return &dudy; case LES_DUDZ: return &dudz;
      case LES_DVDX: return &dvdx; case LES_DVDY: return &dvdy; case LES_DVDZ: return &dvdz;
      case LES_DWDX: return &dwdx; case LES_DWDY: return &dwdy; case LES_DWDZ: return &dwdz;
      case LES_RHSX: return &RHSx; case LES_RHSY: return &RHSy; case LES_RHSZ: return &RHSz;
      case LES_RHSX_F: return &RHSx_f; case LES_RHSY_F: return &RHSy_f; case LES_RHSZ_F: return &RHSz_f;
      case LES_DPDX: return &dpdx; case LES_DPDY: return &dpdy; case LES_DPDZ: return &dpdz;
      case LES_TXX: return &txx; case LES_TXY: return &txy; case LES_TYY: return &tyy;
      case LES_TXZ: return &txz; case LES_TYZ: return &tyz; case LES_TZZ: return &tzz;
      case LES_DIVTX: return &divtx; case LES_DIVTY: return &divty; case LES_DIVTZ: return &divtz;
      case LES_P: return &p;
      case LES_F_LM: return &F_LM; case LES_F_MM: return &F_MM; case LES_F_QN: return &F_QN; case LES_F_NN: return &F_NN;
      case LES_BETA: return &Beta; case LES_CS_OPT2: return &Cs_opt2; case LES_NU_T: return &Nu_t;
      case LES_U_LAG: return &u_lag; case LES_V_LAG: return &v_lag; case LES_W_LAG: return &w_lag;
      case LES_RHS_T: return &RHS_T; case LES_RHS_TF: return &RHS_Tf; case LES_BETA_SCAL: return &beta_scal;
      case LES_DTDX: return &dTdx; case LES_DTDY: return &dTdy; case LES_DTDZ: return &dTdz;
      case LES_S11: return &S11; case LES_S12: return &S12; case LES_S13: return &S13;
      case LES_S22: return &S22; case LES_S23: return &S23; case LES_S33: return &S33;
      case LES_ZO: return &zo; case LES_WT_S: return &wt_s; case LES_USTAR_AVG: return &ustar_avg;
      case LES_PHI_M: return &phi_m; case LES_PSI_M: return &psi_m; case LES_PSI_M0: return &psi_m0;
      case LES_PHI_H: return &phi_h; case LES_PSI_H: return &psi_h; case LES_PSI_H0: return &psi_h0;
      case LES_SGS_T3_SFC: return &sgs_t3;
      case LES_Q: return &qmix; case LES_RHS_Q: return &RHS_q; case LES_RHS_QF: return &RHS_qf;
      case LES_DQDX: return &dqdx; case LES_DQDY: return &dqdy; case LES_DQDZ: return &dqdz;
      case LES_WQ_S: return &wq_s; case LES_SGS_Q3_SFC: return &sgs_q3;
      case LES_G_LM: return &G_LM; case LES_G_MM: return &G_MM; case LES_G_QN: return &G_QN;
      case LES_G_NN: return &G_NN; case LES_PR_T: return &Pr_t; case LES_U_LAG_S: return &u_lag_s;
      case LES_V_LAG_S: return &v_lag_s; case LES_W_LAG_S: return &w_lag_s; case LES_TN_LMMM: return &TnLMMM;
      case LES_TN_QNNN: return &TnQNNN;
      default: return nullptr;
    }
  }
};

}  // namespace les_oracle

using les_oracle::Oracle;

extern "C" {

void* lo_create(const les_config* cfg) {
  try {
    return new Oracle(*cfg);
  } catch (...) {
    return nullptr;
  }
}
void lo_destroy(void* h) { delete (Oracle*)h; }
void lo_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n);
#else
  (void)n;
#endif
}
int lo_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
// Pointer to an internal array and its element count (for numpy views).
double* lo_field(void* h, int id, long* n) {
  Oracle* o = (Oracle*)h;
  les_oracle::Field* f = o->field(id);
  if (!f) { *n = 0; return nullptr; }
  *n = (long)f->size();
  return f->data();
}
void lo_set_surface(void* h, const double* zo, const double* wt_s) {
  Oracle* o = (Oracle*)h;
  for (size_t i = 0; i < o->zo.size(); ++i) {
    o->zo[i] = zo[i];
    o->z_os[i] = zo[i] / 7.39;  // bottombc.f90:274 with zom/z_i = zo
    o->wt_s[i] = wt_s[i];
  }
}
int lo_step(void* h, int nsteps) {
  Oracle* o = (Oracle*)h;
  for (int i = 0; i < nsteps; ++i) {
    int st = o->step();
    if (st != 0) return st;
  }
  return 0;
}
void lo_counters(void* h, int* jt, int* jt_total) { *jt = ((Oracle*)h)->jt; *jt_total = ((Oracle*)h)->jt_total; }
void lo_set_counters(void* h, int jt, int jt_total) { ((Oracle*)h)->jt = jt; ((Oracle*)h)->jt_total = jt_total; }
double lo_rmsdiv(void* h) { return ((Oracle*)h)->rmsdiv(); }
void lo_timestep_conditions(void* h, double* cflu, double* visc) { ((Oracle*)h)->timestep_conditions(cflu, visc); }
// per-routine entry points on caller arrays
void lo_fft_r2c(void* h, double* pl, int nplanes, int big) {
  Oracle* o = (Oracle*)h;
  const size_t np = big ? o->nplane_big : o->nplane;
  for (int i = 0; i < nplanes; ++i) (big ? o->fb : o->fs)->r2c(pl + (size_t)i * np);
}
void lo_fft_c2r(void* h, double* pl, int nplanes, int big) {
  Oracle* o = (Oracle*)h;
  const size_t np = big ? o->nplane_big : o->nplane;
  for (int i = 0; i < nplanes; ++i) (big ? o->fb : o->fs)->c2r(pl + (size_t)i * np);
}
void lo_ddx(void* h, double* df, const double* f, int nlev) { ((Oracle*)h)->ddx(df, f, nlev); }
void lo_ddy(void* h, double* df, const double* f, int nlev) { ((Oracle*)h)->ddy(df, f, nlev); }
void lo_ddxy(void* h, double* dx_, double* dy_, const double* f, int nlev) { ((Oracle*)h)->ddxy(dx_, dy_, f, nlev); }
void lo_filt_da(void* h, double* f, double* dx_, double* dy_, int nlev) { ((Oracle*)h)->filt_da(f, dx_, dy_, nlev); }
void lo_ddz_uv(void* h, double* df, const double* f) { ((Oracle*)h)->ddz_uv(df, f); }
void lo_ddz_w(void* h, double* df, const double* f) { ((Oracle*)h)->ddz_w(df, f); }
void lo_dealias1(void* h, const double* uu, double* ub, int nlev) { ((Oracle*)h)->dealias1(uu, ub, nlev); }
void lo_dealias2(void* h, double* uu, double* ub, int nlev) { ((Oracle*)h)->dealias2(uu, ub, nlev); }
void lo_padd(void* h, double* ub, const double* us) { ((Oracle*)h)->padd(ub, us); }
void lo_unpadd(void* h, double* cc, const double* cb) { ((Oracle*)h)->unpadd(cc, cb); }
void lo_test_filter(void* h, double* f, int which) {
  Oracle* o = (Oracle*)h;
  o->test_filter(f, which == 0 ? o->G_test : o->G_test_test);
}
void lo_filter_G(void* h, double* G, int which) {
  Oracle* o = (Oracle*)h;
  const les_oracle::Field& s = which == 0 ? o->G_test : o->G_test_test;
  std::copy(s.begin(), s.end(), G);
}
void lo_wavenumbers(void* h, double* kx, double* ky) {
  Oracle* o = (Oracle*)h;
  std::copy(o->kx.begin(), o->kx.end(), kx);
  std::copy(o->ky.begin(), o->ky.end(), ky);
}
int lo_tridag_array(void* h, const double* a, const double* b, const double* c, const double* r, double* uu) {
  return ((Oracle*)h)->tridag_array(a, b, c, r, uu);
}
int lo_press_stag_array(void* h, double* p_hat, double* dfdx, double* dfdy) {
  return ((Oracle*)h)->press_stag_array(p_hat, dfdx, dfdy);
}
void lo_convec(void* h, double* cx, double* cy, double* cz) { ((Oracle*)h)->convec(cx, cy, cz); }
void lo_divstress_uv(void* h, double* d, const double* tx, const double* ty, const double* tz) { ((Oracle*)h)->divstress_uv(d, tx, ty, tz); }
void lo_divstress_w(void* h, double* d, const double* tx, const double* ty, const double* tz) { ((Oracle*)h)->divstress_w(d, tx, ty, tz); }
void lo_sgs_stag(void* h) { ((Oracle*)h)->sgs_stag(); }
void lo_calc_sij(void* h) { ((Oracle*)h)->calc_Sij(); }
void lo_lagrange_sdep(void* h) {
  Oracle* o = (Oracle*)h;
  o->lagrange_Sdep(o->S11.data(), o->S12.data(), o->S13.data(), o->S22.data(), o->S23.data(), o->S33.data());
}
void lo_interpolag_sdep(void* h) { ((Oracle*)h)->interpolag_Sdep(); }
void lo_interpolag_ssim(void* h) { ((Oracle*)h)->interpolag_Ssim(); }
void lo_lagrange_ssim(void* h, const double* s11, const double* s12, const double* s13, const double* s22,
                      const double* s23, const double* s33) {
  ((Oracle*)h)->lagrange_Ssim(s11, s12, s13, s22, s23, s33);
}
void lo_scaledep_dynamic(void* h, double* cs_z) {
  Oracle* o = (Oracle*)h;
  o->scaledep_dynamic(cs_z, o->S11.data(), o->S12.data(), o->S13.data(), o->S22.data(), o->S23.data(), o->S33.data());
}
void lo_std_dynamic(void* h, double* cs_z, const double* s11, const double* s12, const double* s13,
                    const double* s22, const double* s23, const double* s33) {
  ((Oracle*)h)->std_dynamic(cs_z, s11, s12, s13, s22, s23, s33);
}
void lo_wallstress(void* h) { ((Oracle*)h)->wallstress(); }
void lo_obukhov(void* h) { ((Oracle*)h)->obukhov(); }
void lo_project(void* h) { ((Oracle*)h)->project(); }
void lo_theta_all_in_one(void* h) { ((Oracle*)h)->theta_all_in_one(); }
void lo_q_all_in_one(void* h) { ((Oracle*)h)->q_all_in_one(); }
void lo_lagrange_scalar_sdep(void* h, double* cs2_pr) {
  Oracle* o = (Oracle*)h;
  o->lagrange_scalar_Sdep(cs2_pr, o->S11.data(), o->S12.data(), o->S13.data(), o->S22.data(), o->S23.data(),
                          o->S33.data());
}
void lo_interpolag_scalar_sdep(void* h) { ((Oracle*)h)->interpolag_scalar_Sdep(); }
void lo_stats_enable(void* h, int c_count, int p_count) { ((Oracle*)h)->stats_enable(c_count, p_count); }
void lo_stats_accumulate(void* h) { ((Oracle*)h)->stats_accumulate(); }
void lo_stats_reset(void* h, int group) { ((Oracle*)h)->stats_reset(group); }
// statistic by name into out (nx,ny,nz-1); 0 if it exists
int lo_stats_get(void* h, const char* name, double* out) {
  Oracle* o = (Oracle*)h;
  for (size_t i = 0; i < o->stat_names.size(); ++i)
    if (o->stat_names[i] == name) {
      std::copy(o->stats[i].begin(), o->stats[i].end(), out);
      return 0;
    }
  return -1;
}
void lo_atm_thermodynamics(void* h, double* o0, double* o1, double* o2, double* o3, double* o4, double* o5,
                           double* o6, double* o7, double* o8) {
  double* o[9] = {o0, o1, o2, o3, o4, o5, o6, o7, o8};
  ((Oracle*)h)->thermo(o);
}

}  // extern "C"
