// Host geometry for a polar-0 case. Every expression keeps the operand order of
// the reference macro it restates, and this file is compiled with
// -ffp-contract=off, so the tables are bit-identical to the values the
// reference computes per cell.
#include <cmath>

#include "sw2g_internal.h"

namespace sw2g {
namespace {

struct Planet {
  double rE, rP, eps2, gE, Omega;
};

double ref_pi() { return 4.0 * std::atan(1.0); }                                   // sw.h:16
double deg2rad(double a) { return a * (ref_pi() / 180.0); }                        // sw.h:108
double linspace_val(int i, double x0, double x1, int n) {                          // tools.c:256-273
  return x0 + (double)i * (x1 - x0) / ((double)n);
}
double rZ(const Planet& p, double lat) {                                           // sw.h:174
  return p.rE / std::sqrt(1.0 + (std::tan(lat) * std::tan(lat)) / p.eps2);
}
double rM(const Planet& p, double lat) {                                           // sw.h:175
  double q = rZ(p, lat) / (p.rE * std::cos(lat));
  return p.rE / p.eps2 * (q * q * q);
}
double lat2pclat(const Planet& p, double lat) { return std::atan(1.0 / p.eps2 * std::tan(lat)); }  // sw.h:170
double radius(const Planet& p, double pc) {                                        // sw.h:172
  double a = p.rE * std::sin(pc), b = p.rP * std::cos(pc);
  return p.rE * p.rP / std::sqrt(a * a + b * b);
}
double g_eff(const Planet& p, double pc) {                                         // sw.h:178-179
  double r = radius(p, pc);
  double g0 = (p.gE + p.Omega * p.Omega * p.rE) * ((p.rE / r) * (p.rE / r));
  return g0 - p.Omega * p.Omega * r * std::cos(pc);
}
double fcor(const Planet& p, double lat) { return 2.0 * p.Omega * std::sin(lat); }  // sw.h:193

// Band limits in radians: as the .sw file gives them (degrees, converted as
// init.c:56-58 does), or already converted (SW2G_FLAG_RADIANS).
double angle(const sw2g_case& c, double a) { return (c.flags & SW2G_FLAG_RADIANS) ? a : deg2rad(a); }

}  // namespace

void build_rows(const sw2g_case& c, std::vector<double>& rows, double* rest_mx, double* rest_my) {
  const int ny = c.ny, H = c.ny + 4;
  Planet p{c.rE, c.rP, (c.rE / c.rP) * (c.rE / c.rP), c.gE, c.Omega};  // init.c:150
  if (c.polar != 0) {
    // init_polar_region (init.c:273-276) turns the spheroid into the sphere of
    // radius rE^2/rP after the gravity and Coriolis fields; epsilon2 keeps its
    // value, so the metric factors below use the new radius with the old ratio
    const double r = (c.rE) * (c.rE) / (c.rP);
    p.rE = r;
    p.rP = r;
  }
  const double lon0 = angle(c, c.lon0), lon1 = angle(c, c.lon1);
  const double lat0 = angle(c, c.lat0), lat1 = angle(c, c.lat1);
  const double dlon = (lon1 - lon0) / ((double)c.nx);                    // coords.c:36
  const double dlat = (lat1 - lat0) / ((double)ny);
  auto latn = [&](int j) { return linspace_val(j, lat0, lat1, ny); };    // sw.h:116
  auto latc = [&](int j) { return (latn(j) + latn(j - 1)) / 2.; };       // sw.h:117
  rows.assign((size_t)R_NUM * H, 0.0);
  auto R = [&](int t, int j) -> double& { return rows[(size_t)t * H + (j + 1)]; };
  const double Dt = c.Dt;
  for (int j = -1; j <= ny + 2; j++) {
    const double lc = latc(j), ln = latn(j);
    R(R_DXE, j) = dlon * rZ(p, lc);                                      // coords.c:60-65
    R(R_DXC, j) = dlon * rZ(p, lc);
    R(R_DXV, j) = dlon * rZ(p, ln);
    R(R_DYN, j) = dlat * rM(p, lc);
    R(R_DYC, j) = dlat * rM(p, latn(j - 1));
    R(R_DYV, j) = dlat * rM(p, lc);
    R(R_GE, j) = g_eff(p, lat2pclat(p, lc));                             // init.c:287-290
    R(R_GN, j) = g_eff(p, lat2pclat(p, ln));
    R(R_GC, j) = g_eff(p, lat2pclat(p, lc));
    R(R_FE, j) = fcor(p, lc);                                            // init.c:292-295
    R(R_FN, j) = fcor(p, ln);
    R(R_RMC, j) = rM(p, lc);
    R(R_RZC, j) = rZ(p, lc);
    R(R_RMN, j) = rM(p, ln);
    R(R_RZN, j) = rZ(p, ln);
    R(R_SINC, j) = std::sin(lc);
    R(R_SINN, j) = std::sin(ln);
  }
  for (int j = -1; j <= ny + 2; j++) {
    R(R_KX, j) = R(R_RMC, j) / R(R_RZC, j);
    R(R_KY, j) = R(R_RZN, j) / R(R_RMN, j);
    R(R_KC, j) = 1.0 / (R(R_RMC, j) * R(R_RZC, j));
    R(R_GEO, j) = Dt * R(R_SINC, j) / R(R_RZC, j);
    R(R_IDXE, j) = 1.0 / R(R_DXE, j);
    R(R_IDXC, j) = 1.0 / R(R_DXC, j);
    R(R_IDXV, j) = 1.0 / R(R_DXV, j);
    R(R_IDYN, j) = 1.0 / R(R_DYN, j);
    R(R_IDYC, j) = 1.0 / R(R_DYC, j);
    R(R_DTFE, j) = Dt * R(R_FE, j);
    R(R_DTFN, j) = Dt * R(R_FN, j);
    R(R_MGEDT, j) = -R(R_GE, j) * Dt;
    R(R_MGNDT, j) = -R(R_GN, j) * Dt;
    R(R_DXE2, j) = R(R_DXE, j) + R(R_DXE, j);
    R(R_DYNS, j) = (j + 1 <= ny + 2) ? R(R_DYN, j) + R(R_DYN, j + 1) : 0.0;
    R(R_SURF, j) = R(R_DXC, j) * R(R_DYC, j);
    R(R_IDYV, j) = 1.0 / R(R_DYV, j);
    R(R_IDXE2, j) = 1.0 / R(R_DXE2, j);
    R(R_IDYNS, j) = (j + 1 <= ny + 2) ? 1.0 / R(R_DYNS, j) : 0.0;
    R(R_IRZC, j) = 1.0 / R(R_RZC, j);
    R(R_IRZN, j) = 1.0 / R(R_RZN, j);
  }
  // compute_Dt fallback for a flow at rest (calc.c:715-725): depends on geometry only
  double mx = 0, my = 0;
  for (int j = 1; j <= ny; j++) {
    double cx = std::sqrt((c.depth) * (R(R_GE, j))), cy = std::sqrt((c.depth) * (R(R_GN, j)));
    if (std::fabs(cx / R(R_DXE, j)) > mx) mx = std::fabs(cx) / R(R_DXE, j);
    if (std::fabs(cy / R(R_DYN, j)) > my) my = std::fabs(cy) / R(R_DYN, j);
  }
  *rest_mx = mx;
  *rest_my = my;
}

namespace {
double great_angle(double lon0, double lat0, double lon1, double lat1) {  // tools.c:122-136
  return std::acos(std::sin(lat0) * std::sin(lat1) + std::cos(lat0) * std::cos(lat1) * std::cos(lon1 - lon0));
}
}  // namespace

void polar_fields(const sw2g_case& c, std::vector<double>& f, double* rest_mx, double* rest_my) {
  const int nx = c.nx, ny = c.ny, W = nx + 4, Hh = ny + 4;
  const size_t S = (size_t)W * Hh;
  f.assign((size_t)P_NUM * S, 0.0);
  // init_polar_region runs on the spheroid as read (init.c:243-271)
  const Planet p{c.rE, c.rP, (c.rE / c.rP) * (c.rE / c.rP), c.gE, c.Omega};
  const double lon0 = angle(c, c.lon0), lon1 = angle(c, c.lon1);
  const double lat0 = angle(c, c.lat0), lat1 = angle(c, c.lat1);
  const double beta = angle(c, c.beta_sponge);
  const double mlon = ((lon0) + (lon1)) / 2.0, mlat = ((lat0) + (lat1)) / 2.0;  // MEAN, sw.h:110
  const double pi = ref_pi(), ns = (double)c.polar;
  const double tau_sponge = -std::log(0.01) / (std::sqrt(2.0) * lat1 - beta);  // init.c:157
  const double sigma_dis = (c.flags & SW2G_FLAG_SIGMA) ? c.tau : (c.tau > 1e10 ? 0 : 1.0 / c.tau);
  auto lone = [&](int i) { return linspace_val(i, lon0, lon1, nx); };       // sw.h:113
  auto lonc = [&](int i) { return (lone(i) + lone(i - 1)) / 2.; };          // sw.h:114
  auto latn = [&](int j) { return linspace_val(j, lat0, lat1, ny); };       // sw.h:116
  auto latc = [&](int j) { return (latn(j) + latn(j - 1)) / 2.; };          // sw.h:117
  auto polar_lat = [&](double lon, double lat) {                            // sw.h:130-132
    return (ns) * (pi / 2.0 - great_angle(lon, lat, mlon, mlat));
  };
  auto sponge = [&](double lon, double lat, double outside) {               // calc.c:102-111, 378-392
    const double dist = great_angle(mlon, mlat, lon, lat) - beta;
    return (dist > 0) ? c.sigma_sponge * (1.0 - std::exp(-tau_sponge * (dist))) : outside;
  };
  auto F = [&](int t, int i, int j) -> double& { return f[(size_t)t * S + (i + 1) + (size_t)(j + 1) * W]; };
  for (int j = -1; j <= ny + 2; j++)
    for (int i = -1; i <= nx + 2; i++) {
      const double le = polar_lat(lone(i), latc(j)), ln = polar_lat(lonc(i), latn(j));
      const double lc = polar_lat(lonc(i), latc(j));
      F(P_GE, i, j) = g_eff(p, lat2pclat(p, le));                           // init.c:253-261
      F(P_GN, i, j) = g_eff(p, lat2pclat(p, ln));
      F(P_GC, i, j) = g_eff(p, lat2pclat(p, lc));
      F(P_FE, i, j) = fcor(p, le);
      F(P_FN, i, j) = fcor(p, ln);
      F(P_SH, i, j) = sponge(lonc(i), latc(j), sigma_dis);
      F(P_STR, i, j) = sponge(lonc(i), latc(j), c.tracer_dis);
      F(P_SU, i, j) = sponge(lone(i), latc(j), sigma_dis);
      F(P_SV, i, j) = sponge(lonc(i), latn(j), sigma_dis);
    }
  // compute_Dt for a flow at rest (calc.c:715-725) with these gravity fields
  // and the metric factors of the sphere
  std::vector<double> rows;
  double mx0 = 0, my0 = 0;
  build_rows(c, rows, &mx0, &my0);
  const int H = ny + 4;
  double mx = 0, my = 0;
  for (int j = 1; j <= ny; j++) {
    const double dxe = rows[(size_t)R_DXE * H + j + 1], dyn = rows[(size_t)R_DYN * H + j + 1];
    for (int i = 1; i <= nx; i++) {
      const double cx = std::sqrt((c.depth) * (F(P_GE, i, j))), cy = std::sqrt((c.depth) * (F(P_GN, i, j)));
      if (std::fabs(cx / dxe) > mx) mx = std::fabs(cx) / dxe;
      if (std::fabs(cy / dyn) > my) my = std::fabs(cy) / dyn;
    }
  }
  *rest_mx = mx;
  *rest_my = my;
}

// Area element DXC*DYC and gravity GC of interior rows j0..j0+n-1 (the two
// per-row values the energy sum needs), into caller-owned arrays; uses the
// same expressions as build_rows and allocates nothing.
void energy_row_geometry(const sw2g_case& c, int j0, int n, double* surf, double* gc) {
  Planet p{c.rE, c.rP, (c.rE / c.rP) * (c.rE / c.rP), c.gE, c.Omega};
  const double lon0 = angle(c, c.lon0), lon1 = angle(c, c.lon1);
  const double lat0 = angle(c, c.lat0), lat1 = angle(c, c.lat1);
  const double dlon = (lon1 - lon0) / ((double)c.nx);
  const double dlat = (lat1 - lat0) / ((double)c.ny);
  for (int q = 0; q < n; q++) {
    const int j = j0 + q;
    const double ln1 = linspace_val(j - 1, lat0, lat1, c.ny), ln = linspace_val(j, lat0, lat1, c.ny);
    const double lc = (ln + ln1) / 2.;
    const double dxc = dlon * rZ(p, lc), dyc = dlat * rM(p, ln1);
    surf[q] = dxc * dyc;
    gc[q] = g_eff(p, lat2pclat(p, lc));
  }
}

double forcing_lon_span(const sw2g_case& c) { return angle(c, c.lon1) - angle(c, c.lon0); }

double forcing_pclat(const sw2g_case& c, double lat) {
  const Planet p{c.rE, c.rP, (c.rE / c.rP) * (c.rE / c.rP), c.gE, c.Omega};
  return lat2pclat(p, lat);
}

void forcing_tables(const sw2g_case& c, std::vector<double>& rows3, std::vector<double>& pl,
                    std::vector<double>& lonc) {
  const Planet p{c.rE, c.rP, (c.rE / c.rP) * (c.rE / c.rP), c.gE, c.Omega};
  const double lon0 = angle(c, c.lon0), lon1 = angle(c, c.lon1);
  const double lat0 = angle(c, c.lat0), lat1 = angle(c, c.lat1);
  const double dlon = (lon1 - lon0) / ((double)c.nx);                    // coords.c:60-65
  const double dlat = (lat1 - lat0) / ((double)c.ny);
  auto latn = [&](int j) { return linspace_val(j, lat0, lat1, c.ny); };  // sw.h:116
  auto latc = [&](int j) { return (latn(j) + latn(j - 1)) / 2.; };       // sw.h:117
  auto lone = [&](int i) { return linspace_val(i, lon0, lon1, c.nx); };  // sw.h:113
  rows3.assign(3 * (size_t)(c.ny + 2), 0.0);
  pl.assign((size_t)c.ny + 2, 0.0);
  lonc.assign((size_t)c.nx + 2, 0.0);
  for (int j = 0; j <= c.ny + 1; j++) {
    const double pc = lat2pclat(p, latc(j));
    pl[j] = pc;
    rows3[3 * j] = std::sin(pc);
    rows3[3 * j + 1] = std::cos(pc);
    rows3[3 * j + 2] = (dlon * rZ(p, latc(j))) * (dlat * rM(p, latn(j - 1)));  // DXC * DYC
  }
  for (int i = 0; i <= c.nx + 1; i++) lonc[i] = (lone(i) + lone(i - 1)) / 2.;  // sw.h:114
}

}  // namespace sw2g
