// Running statistics of io.f90:403-1218 (MM_XYZ_Out) on the device.
//
// 133 FP64 accumulators of nx ny (nz-1) points, statistic s of point
// (jx, jy, k) at stats[s * S + jx + nx (jy + ny (k - 1))], S = nx ny (nz-1).
// One kernel thread per point forms the w-node interpolated quantities of
// io.f90:528-624 (arg1..arg8, the averaged gradients, the pressure
// gradients corrected by the advective terms), the thermodynamic
// diagnostics of atm_thermodynamics.f90:37-52 at the point, and adds
// fr * (product) to every accumulator (io.f90:628-831).
#include <cmath>
#include <cstring>

#include "common.cuh"
#include "les_internal.h"

namespace les {

// accumulator order, names after the reference's arrays, and the group
// each is written and zeroed with: 1 every p_count steps (io.f90:966-1006),
// 2 every 2 p_count steps (io.f90:1009-1216), 0 never (atxy)
enum StatId {
  ST_AACTUAL_T, ST_AACTUAL_TV, ST_APR_ATM, ST_AREL_HUM, ST_AREL_HUM_Q, ST_AVAPOR_PR, ST_ASAT_VAPOR_PR,
  ST_ASAT_QMIX, ST_AZLCL_ALL,
  ST_AU, ST_AV, ST_AW, ST_AP, ST_ATHETA, ST_AQ,
  ST_U2, ST_V2, ST_W2, ST_P2, ST_THETA2, ST_Q2, ST_TKE, ST_U3, ST_V3, ST_W3, ST_T3, ST_Q3,
  ST_AWE, ST_AVE, ST_AUE, ST_AUW, ST_AVW, ST_AWT, ST_AWQ, ST_AUV, ST_AUT, ST_AVT, ST_AUQ, ST_AVQ,
  ST_AWUU, ST_AWVV, ST_AWTT, ST_AWQQ, ST_AWWU, ST_AWWV, ST_AWWT, ST_AWWQ,
  ST_ASGST3, ST_ASGSQ3,
  ST_ADUDX, ST_ADUDY, ST_ADUDZ, ST_ADVDX, ST_ADVDY, ST_ADVDZ, ST_ADWDX, ST_ADWDY, ST_ADWDZ,
  ST_ADTDX, ST_ADTDY, ST_ADTDZ, ST_ADQDX, ST_ADQDY, ST_ADQDZ, ST_ADPDX, ST_ADPDY, ST_ADPDZ,
  ST_ATXX, ST_ATXY, ST_ATXZ, ST_ATYZ, ST_ATYY, ST_ATZZ,
  ST_AUP, ST_AVP, ST_AWP, ST_ATP, ST_AQP, ST_ATQ, ST_AUPX, ST_AUPY, ST_AUPZ, ST_AVPX, ST_AVPY, ST_AVPZ,
  ST_AWPX, ST_AWPY, ST_AWPZ,
  ST_AT11UX, ST_AT12UY, ST_AT13UZ, ST_AT21VX, ST_AT22VY, ST_AT23VZ, ST_AT31WX, ST_AT32WY, ST_AT33WZ,
  ST_APUX, ST_APUY, ST_APUZ, ST_APVX, ST_APVY, ST_APVZ, ST_APWX, ST_APWY, ST_APWZ, ST_APTX, ST_APTY, ST_APTZ,
  ST_APQX, ST_APQY, ST_APQZ,
  ST_AS11, ST_AS12, ST_AS13, ST_AS22, ST_AS23, ST_AS33,
  ST_AT11S11, ST_AT12S12, ST_AT13S13, ST_AT22S22, ST_AT23S23, ST_AT33S33,
  ST_AUT11, ST_AUT12, ST_AUT13, ST_AVT21, ST_AVT22, ST_AVT23, ST_AWT31, ST_AWT32, ST_AWT33,
  ST_COUNT
};
static const char* const kStatName[ST_COUNT] = {
    "aactual_T", "aactual_Tv", "apr_atm", "arel_hum", "arel_hum_q", "avapor_pr", "asat_vapor_pr",
    "asat_qmix", "azlcl_all",
    "au", "av", "aw", "ap", "atheta", "aq",
    "u2", "v2", "w2", "p2", "theta2", "q2", "tke", "u3", "v3", "w3", "T3", "q3",
    "awe", "ave", "aue", "auw", "avw", "awt", "awq", "auv", "aut", "avt", "auq", "avq",
    "awuu", "awvv", "awtt", "awqq", "awwu", "awwv", "awwt", "awwq",
    "asgst3", "asgsq3",
    "adudx", "adudy", "adudz", "advdx", "advdy", "advdz", "adwdx", "adwdy", "adwdz",
    "adTdx", "adTdy", "adTdz", "adqdx", "adqdy", "adqdz", "adpdx", "adpdy", "adpdz",
    "atxx", "atxy", "atxz", "atyz", "atyy", "atzz",
    "aup", "avp", "awp", "atp", "aqp", "atq", "aupx", "aupy", "aupz", "avpx", "avpy", "avpz",
    "awpx", "awpy", "awpz",
    "at11ux", "at12uy", "at13uz", "at21vx", "at22vy", "at23vz", "at31wx", "at32wy", "at33wz",
    "apux", "apuy", "apuz", "apvx", "apvy", "apvz", "apwx", "apwy", "apwz", "aptx", "apty", "aptz",
    "apqx", "apqy", "apqz",
    "as11", "as12", "as13", "as22", "as23", "as33",
    "at11s11", "at12s12", "at13s13", "at22s22", "at23s23", "at33s33",
    "aut11", "aut12", "aut13", "avt21", "avt22", "avt23", "awt31", "awt32", "awt33"};
static int stat_group(int s) {
  switch (s) {
    case ST_AU: case ST_AV: case ST_AW: case ST_ATHETA: case ST_AQ: case ST_U2: case ST_V2: case ST_W2:
    case ST_THETA2: case ST_Q2: case ST_AUW: case ST_AVW: case ST_AWT: case ST_AWQ: case ST_ATXZ:
    case ST_ATYZ: case ST_ASGST3: case ST_ASGSQ3: case ST_AZLCL_ALL:
      return 1;
    case ST_ATXY:
      return 0;
    default:
      return 2;
  }
}

// the module arrays the accumulation reads; NT: storage of the fields an
// FP32-mixed context holds in FP32 (horizontal gradients, tau, Nu_t)
template <typename NT> struct StatsIn {
  const double *u, *v, *w, *theta, *q, *p;
  const NT *dudx, *dudy, *dvdx, *dvdy, *dwdx, *dwdy;
  const double *dudz, *dvdz, *dwdz;
  const NT *dTdx, *dTdy, *dqdx, *dqdy;
  const double *dTdz, *dqdz;
  const double *dpdx, *dpdy, *dpdz;
  const NT *txx, *txy, *txz, *tyy, *tyz, *tzz, *nut;
  const double *sgs_t3, *sgs_q3;  // surface planes (nx,ny); sgs_q3 null without humidity
};
template <typename NT> __device__ __forceinline__ double ld(const NT* p, size_t i) { return cvt<double, NT>(p[i]); }

// grid (ceil(ld ny / 256), nz - 1)
template <typename NT>
__global__ void __launch_bounds__(256) k_stats(StatsIn<NT> in, double* __restrict__ acc, int ld_, int nx, int ny,
                                               int nz, double fr, double pr, double dz, double z_i, double T_scale,
                                               double q_scale, double g) {
  const unsigned np = (unsigned)ld_ * ny;
  const unsigned r = blockIdx.x * 256u + threadIdx.x;
  if (r >= np) return;
  const int jy = (int)(r / (unsigned)ld_), jx = (int)(r - (unsigned)jy * ld_);
  if (jx >= nx) return;
  const int k = blockIdx.y + 1;  // 1..nz-1
  const size_t i = (size_t)(k - 1) * np + r, im = i - np, ip = i + np;
  const size_t S = (size_t)nx * ny * (nz - 1);
  double* a = acc + (size_t)jx + (size_t)nx * ((size_t)jy + (size_t)ny * (k - 1));
  auto add = [&](int s, double val) { a[(size_t)s * S] = a[(size_t)s * S] + val; };
  const bool hq = in.q != nullptr;
  const double qk = hq ? in.q[i] : 0.0;
  // io.f90:528-624
  double a1, a2, a3, a4, a7, a8, ux, uy, uz, vx, vy, vz, wx, wy, wz, px, py, pz, tx, ty, tz, qx, qy, qz;
  const size_t pk = (size_t)k * np + r, pkm = pk - np;  // p(ld,ny,0:nz)
  if (k == 1) {
    a1 = in.u[i];
    a2 = in.v[i];
    a3 = 0.25 * in.w[ip];
    a4 = in.p[pk] - 0.5 * (a1 * a1 + a2 * a2 + a3 * a3);
    a7 = in.theta[i];
    a8 = qk;
    ux = ld(in.dudx, i); uy = ld(in.dudy, i); uz = in.dudz[i];
    vx = ld(in.dvdx, i); vy = ld(in.dvdy, i); vz = in.dvdz[i];
    wx = ld(in.dwdx, ip) / 2.0; wy = ld(in.dwdy, ip) / 2.0; wz = in.dwdz[i];
    px = in.dpdx[i] - a1 * ux - a2 * vx - a3 * wx;
    py = in.dpdy[i] - a1 * uy - a2 * vy - a3 * wy;
    pz = in.dpdz[i] - a1 * uz - a2 * vz - a3 * wz;
    tx = ld(in.dTdx, i); ty = ld(in.dTdy, i); tz = in.dTdz[i];
    qx = hq ? ld(in.dqdx, i) : 0.0; qy = hq ? ld(in.dqdy, i) : 0.0; qz = hq ? in.dqdz[i] : 0.0;
  } else {
    a1 = (in.u[i] + in.u[im]) / 2.0;
    a2 = (in.v[i] + in.v[im]) / 2.0;
    a3 = in.w[i];
    a4 = ((in.p[pk] + in.p[pkm]) / 2.0 - 0.5 * (a1 * a1 + a2 * a2 + a3 * a3));
    a7 = (in.theta[i] + in.theta[im]) / 2.0;
    a8 = hq ? (in.q[i] + in.q[im]) / 2.0 : 0.0;
    ux = (ld(in.dudx, i) + ld(in.dudx, im)) / 2.0; uy = (ld(in.dudy, i) + ld(in.dudy, im)) / 2.0; uz = in.dudz[i];
    vx = (ld(in.dvdx, i) + ld(in.dvdx, im)) / 2.0; vy = (ld(in.dvdy, i) + ld(in.dvdy, im)) / 2.0; vz = in.dvdz[i];
    wx = ld(in.dwdx, i); wy = ld(in.dwdy, i); wz = (in.dwdz[i] + in.dwdz[im]) / 2.0;
    px = (in.dpdx[i] + in.dpdx[im]) / 2.0 - a1 * ux - a2 * vx - a3 * wx;
    py = (in.dpdy[i] + in.dpdy[im]) / 2.0 - a1 * uy - a2 * vy - a3 * wy;
    pz = in.dpdz[i] - a1 * uz - a2 * vz - a3 * wz;
    tx = (ld(in.dTdx, i) + ld(in.dTdx, im)) / 2.0; ty = (ld(in.dTdy, i) + ld(in.dTdy, im)) / 2.0; tz = in.dTdz[i];
    if (hq) {
      qx = (ld(in.dqdx, i) + ld(in.dqdx, im)) / 2.0; qy = (ld(in.dqdy, i) + ld(in.dqdy, im)) / 2.0; qz = in.dqdz[i];
    } else {
      qx = 0.0; qy = 0.0; qz = 0.0;
    }
  }
  // thermodynamics at the point (atm_thermodynamics.f90:37-52, k_global = k)
  {
    const double cp = 1005.0, Rd = 287.04, pr_surf = 100000.0;
    const double zg = k * dz * z_i;
    const double T = in.theta[i] - (g / cp) * zg / T_scale;
    const double Tv = T * (1 + 0.61 * 0.001 * qk * q_scale);
    const double Tc = T * T_scale - 273.2;
    const double es = 611.2 * exp(17.62 * Tc / (243.12 + Tc));
    const double pa = pr_surf * exp(-zg / (Rd * Tv * T_scale / g));
    const double qq = 0.001 * q_scale * qk;
    const double e = (qq / (qq + 0.622)) * pa;
    const double qs = 0.622 * es / (pa - es);
    const double rq = qq / qs;
    const double zl = zg + (cp / g) * (T * T_scale - 55 - 1.0 / (1 / (T * T_scale - 55) - log(rq) / 2840));
    add(ST_AACTUAL_T, fr * T * T_scale);
    add(ST_AACTUAL_TV, fr * Tv * T_scale);
    add(ST_APR_ATM, fr * pa);
    add(ST_AREL_HUM, fr * (e / es));
    add(ST_AREL_HUM_Q, fr * rq);
    add(ST_AVAPOR_PR, fr * e);
    add(ST_ASAT_VAPOR_PR, fr * es);
    add(ST_ASAT_QMIX, fr * qs);
    add(ST_AZLCL_ALL, fr * zl);
  }
  // io.f90:642-717
  add(ST_AU, fr * a1); add(ST_AV, fr * a2); add(ST_AW, fr * a3); add(ST_AP, fr * a4);
  add(ST_ATHETA, fr * a7); add(ST_AQ, fr * a8);
  add(ST_U2, fr * a1 * a1); add(ST_V2, fr * a2 * a2); add(ST_W2, fr * a3 * a3); add(ST_P2, fr * a4 * a4);
  add(ST_THETA2, fr * a7 * a7); add(ST_Q2, fr * a8 * a8);
  const double ke = 0.5 * (a1 * a1 + a2 * a2 + a3 * a3);
  add(ST_TKE, fr * ke);
  add(ST_U3, fr * a1 * a1 * a1); add(ST_V3, fr * a2 * a2 * a2); add(ST_W3, fr * a3 * a3 * a3);
  add(ST_T3, fr * a7 * a7 * a7); add(ST_Q3, fr * a8 * a8 * a8);
  add(ST_AWE, fr * a3 * ke); add(ST_AVE, fr * a2 * ke); add(ST_AUE, fr * a1 * ke);
  add(ST_AUW, fr * a1 * a3); add(ST_AVW, fr * a2 * a3); add(ST_AWT, fr * a3 * a7); add(ST_AWQ, fr * a3 * a8);
  add(ST_AUV, fr * a1 * a2); add(ST_AUT, fr * a1 * a7); add(ST_AVT, fr * a2 * a7); add(ST_AUQ, fr * a1 * a8);
  add(ST_AVQ, fr * a2 * a8);
  add(ST_AWUU, fr * a3 * a1 * a1); add(ST_AWVV, fr * a3 * a2 * a2); add(ST_AWTT, fr * a3 * a7 * a7);
  add(ST_AWQQ, fr * a3 * a8 * a8); add(ST_AWWU, fr * a3 * a3 * a1); add(ST_AWWV, fr * a3 * a3 * a2);
  add(ST_AWWT, fr * a3 * a3 * a7); add(ST_AWWQ, fr * a3 * a3 * a8);
  // the vertical SGS fluxes: the surface flux at level 1, else -Nu_t/Pr d/dz
  // (scalars_module.f90:414-425, scalars_module_q.f90:323-336)
  const size_t s2 = (size_t)jy * nx + jx;
  const double nu = ld(in.nut, i);
  add(ST_ASGST3, fr * (k == 1 ? in.sgs_t3[s2] : -1.0 * ((1.0 / pr) * nu * in.dTdz[i])));
  add(ST_ASGSQ3, fr * (!hq ? 0.0 : (k == 1 ? in.sgs_q3[s2] : -1.0 * ((1.0 / pr) * nu * in.dqdz[i]))));
  // io.f90:751-773
  add(ST_ADUDX, fr * ux); add(ST_ADUDY, fr * uy); add(ST_ADUDZ, fr * uz);
  add(ST_ADVDX, fr * vx); add(ST_ADVDY, fr * vy); add(ST_ADVDZ, fr * vz);
  add(ST_ADWDX, fr * wx); add(ST_ADWDY, fr * wy); add(ST_ADWDZ, fr * wz);
  add(ST_ADTDX, fr * tx); add(ST_ADTDY, fr * ty); add(ST_ADTDZ, fr * tz);
  add(ST_ADQDX, fr * qx); add(ST_ADQDY, fr * qy); add(ST_ADQDZ, fr * qz);
  add(ST_ADPDX, fr * px); add(ST_ADPDY, fr * py); add(ST_ADPDZ, fr * pz);
  // io.f90:778-802
  const double t11 = ld(in.txx, i), t12 = ld(in.txy, i), t13 = ld(in.txz, i);
  const double t22 = ld(in.tyy, i), t23 = ld(in.tyz, i), t33 = ld(in.tzz, i);
  add(ST_ATXX, fr * t11); add(ST_ATXY, fr * t12); add(ST_ATXZ, fr * t13);
  add(ST_ATYZ, fr * t23); add(ST_ATYY, fr * t22); add(ST_ATZZ, fr * t33);
  add(ST_AUP, fr * a1 * a4); add(ST_AVP, fr * a2 * a4); add(ST_AWP, fr * a3 * a4); add(ST_ATP, fr * a7 * a4);
  add(ST_AQP, fr * a8 * a4); add(ST_ATQ, fr * a7 * a8);
  add(ST_AUPX, fr * a1 * px); add(ST_AUPY, fr * a1 * py); add(ST_AUPZ, fr * a1 * pz);
  add(ST_AVPX, fr * a2 * px); add(ST_AVPY, fr * a2 * py); add(ST_AVPZ, fr * a2 * pz);
  add(ST_AWPX, fr * a3 * px); add(ST_AWPY, fr * a3 * py); add(ST_AWPZ, fr * a3 * pz);
  // io.f90:805-846: SGS stress times the raw level-k gradients
  add(ST_AT11UX, fr * t11 * ld(in.dudx, i)); add(ST_AT12UY, fr * t12 * ld(in.dudy, i));
  add(ST_AT13UZ, fr * t13 * in.dudz[i]);
  add(ST_AT21VX, fr * t12 * ld(in.dvdx, i)); add(ST_AT22VY, fr * t22 * ld(in.dvdy, i));
  add(ST_AT23VZ, fr * t23 * in.dvdz[i]);
  add(ST_AT31WX, fr * t13 * ld(in.dwdx, i)); add(ST_AT32WY, fr * t23 * ld(in.dwdy, i));
  add(ST_AT33WZ, fr * t33 * in.dwdz[i]);
  add(ST_APUX, fr * a4 * ux); add(ST_APUY, fr * a4 * uy); add(ST_APUZ, fr * a4 * uz);
  add(ST_APVX, fr * a4 * vx); add(ST_APVY, fr * a4 * vy); add(ST_APVZ, fr * a4 * vz);
  add(ST_APWX, fr * a4 * wx); add(ST_APWY, fr * a4 * wy); add(ST_APWZ, fr * a4 * wz);
  add(ST_APTX, fr * a4 * tx); add(ST_APTY, fr * a4 * ty); add(ST_APTZ, fr * a4 * tz);
  add(ST_APQX, fr * a4 * qx); add(ST_APQY, fr * a4 * qy); add(ST_APQZ, fr * a4 * qz);
  // io.f90:851-876
  const double S11 = ux, S12 = 0.5 * (uy + vx), S13 = 0.5 * (uz + wx), S22 = vy, S23 = 0.5 * (vz + wy), S33 = wz;
  add(ST_AS11, fr * S11); add(ST_AS12, fr * S12); add(ST_AS13, fr * S13);
  add(ST_AS22, fr * S22); add(ST_AS23, fr * S23); add(ST_AS33, fr * S33);
  add(ST_AT11S11, fr * t11 * S11); add(ST_AT12S12, fr * t12 * S12); add(ST_AT13S13, fr * t13 * S13);
  add(ST_AT22S22, fr * t22 * S22); add(ST_AT23S23, fr * t23 * S23); add(ST_AT33S33, fr * t33 * S33);
  add(ST_AUT11, fr * t11 * a1); add(ST_AUT12, fr * t12 * a1); add(ST_AUT13, fr * t13 * a1);
  add(ST_AVT21, fr * t12 * a2); add(ST_AVT22, fr * t22 * a2); add(ST_AVT23, fr * t23 * a2);
  add(ST_AWT31, fr * t13 * a3); add(ST_AWT32, fr * t23 * a3); add(ST_AWT33, fr * t33 * a3);
}

template <typename NT> static StatsIn<NT> stats_in(les_ctx* c) {
  auto F = [&](int f) { return reinterpret_cast<const NT*>(c->f[f]); };
  StatsIn<NT> in;
  in.u = c->f[LES_U]; in.v = c->f[LES_V]; in.w = c->f[LES_W]; in.theta = c->f[LES_THETA];
  in.q = c->cfg.q_flag ? c->f[LES_Q] : nullptr;
  in.p = c->f[LES_P];
  in.dudx = F(LES_DUDX); in.dudy = F(LES_DUDY); in.dvdx = F(LES_DVDX); in.dvdy = F(LES_DVDY);
  in.dwdx = F(LES_DWDX); in.dwdy = F(LES_DWDY);
  in.dudz = c->f[LES_DUDZ]; in.dvdz = c->f[LES_DVDZ]; in.dwdz = c->f[LES_DWDZ];
  in.dTdx = F(LES_DTDX); in.dTdy = F(LES_DTDY);
  in.dqdx = c->cfg.q_flag ? F(LES_DQDX) : nullptr; in.dqdy = c->cfg.q_flag ? F(LES_DQDY) : nullptr;
  in.dTdz = c->f[LES_DTDZ]; in.dqdz = c->cfg.q_flag ? c->f[LES_DQDZ] : nullptr;
  in.dpdx = c->f[LES_DPDX]; in.dpdy = c->f[LES_DPDY]; in.dpdz = c->f[LES_DPDZ];
  in.txx = F(LES_TXX); in.txy = F(LES_TXY); in.txz = F(LES_TXZ); in.tyy = F(LES_TYY); in.tyz = F(LES_TYZ);
  in.tzz = F(LES_TZZ); in.nut = F(LES_NU_T);
  in.sgs_t3 = c->f[LES_SGS_T3_SFC];
  in.sgs_q3 = c->cfg.q_flag ? c->f[LES_SGS_Q3_SFC] : nullptr;
  return in;
}

static size_t stats_elems(const les_ctx* c) { return (size_t)c->g.nx * c->g.ny * (c->g.nz - 1); }

int op_stats(les_ctx* c) {
  const Grid& g = c->g;
  const les_config& k = c->cfg;
  const size_t S = stats_elems(c);
  if (c->jt_total <= c->stats_c) {  // io.f90:457-502: everything but atxy starts from zero
    for (int s = 0; s < ST_COUNT; ++s)
      if (s != ST_ATXY) LES_CUDA_CHECK(cudaMemsetAsync(c->stats + (size_t)s * S, 0, S * sizeof(double), c->stream));
  }
  const double fr = (1.0 / (double)c->stats_p) * (double)c->stats_c;  // io.f90:504
  const dim3 grid((unsigned)((g.nplane + 255) / 256), (unsigned)(g.nz - 1));
  if (k.precision == 1)
    k_stats<float><<<grid, 256, 0, c->stream>>>(stats_in<float>(c), c->stats, g.ld, g.nx, g.ny, g.nz, fr, k.pr, g.dz,
                                                k.z_i, k.t_scale, k.q_scale, k.g);
  else
    k_stats<double><<<grid, 256, 0, c->stream>>>(stats_in<double>(c), c->stats, g.ld, g.nx, g.ny, g.nz, fr, k.pr,
                                                 g.dz, k.z_i, k.t_scale, k.q_scale, k.g);
  LES_COUNT_LAUNCH();
  return 0;
}

}  // namespace les

using namespace les;

extern "C" {

int les_stats_count(void) { return ST_COUNT; }
const char* les_stats_name(int i) { return (i >= 0 && i < ST_COUNT) ? kStatName[i] : nullptr; }
int les_stats_group(int i) { return (i >= 0 && i < ST_COUNT) ? stat_group(i) : -1; }

int les_stats_enable(les_ctx* c, int c_count, int p_count, int auto_accumulate) {
  if (!c || c_count < 1 || p_count < 1) return LES_ERR_ARG;
  if (!c->cfg.s_flag) { les_set_error("running statistics need s_flag = 1 (io.f90:211-213)"); return LES_ERR_STATE; }
  const size_t S = stats_elems(c);
  if (!c->stats) {
    void* p = nullptr;
    if (cudaMalloc(&p, (size_t)ST_COUNT * S * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      les_set_error("cannot allocate the %d running statistics (%zu bytes)", (int)ST_COUNT,
                    (size_t)ST_COUNT * S * sizeof(double));
      return LES_ERR_OOM;
    }
    c->stats = static_cast<double*>(p);
    c->allocs.push_back(p);
    c->bytes += (size_t)ST_COUNT * S * sizeof(double);
  }
  LES_CUDA_CHECK(cudaMemsetAsync(c->stats, 0, (size_t)ST_COUNT * S * sizeof(double), c->stream));
  LES_CUDA_CHECK(cudaStreamSynchronize(c->stream));
  c->stats_c = c_count;
  c->stats_p = p_count;
  c->stats_auto = auto_accumulate ? 1 : 0;
  return LES_OK;
}

int les_stats_accumulate(les_ctx* c) {
  if (!c) return LES_ERR_ARG;
  if (!c->stats) { les_set_error("les_stats_enable first"); return LES_ERR_STATE; }
  op_stats(c);
  LES_CUDA_CHECK(cudaStreamSynchronize(c->stream));
  return LES_OK;
}

int les_stats_get(les_ctx* c, int i, double* host) {
  if (!c || !host || i < 0 || i >= ST_COUNT) return LES_ERR_ARG;
  if (!c->stats) { les_set_error("les_stats_enable first"); return LES_ERR_STATE; }
  const size_t S = stats_elems(c);
  LES_CUDA_CHECK(cudaMemcpyAsync(host, c->stats + (size_t)i * S, S * sizeof(double), cudaMemcpyDeviceToHost,
                                 c->stream));
  LES_CUDA_CHECK(cudaStreamSynchronize(c->stream));
  return LES_OK;
}

int les_stats_reset(les_ctx* c, int group) {
  if (!c || (group != 1 && group != 2)) return LES_ERR_ARG;
  if (!c->stats) { les_set_error("les_stats_enable first"); return LES_ERR_STATE; }
  const size_t S = stats_elems(c);
  for (int s = 0; s < ST_COUNT; ++s)
    if (stat_group(s) == group)
      LES_CUDA_CHECK(cudaMemsetAsync(c->stats + (size_t)s * S, 0, S * sizeof(double), c->stream));
  LES_CUDA_CHECK(cudaStreamSynchronize(c->stream));
  return LES_OK;
}

}  // extern "C"
