// dvm_vis.cpp -- the reference's Tecplot output (input_output/visualization.f90) for one
// monatomic species: the file headers (write_headers :514-762), the macroscopic properties
// (write_properties :1591-1716 with get_data_to_output :2296-2633) and the distribution
// function at chosen cells (write_df :920-1230). Host code only: the caller passes the
// properties it downloaded and, for the columns the reference computes from phi, f.
//
// When f is given, every property is formed from it on the host the way the reference's
// calculate_physical_properties forms it (dist_funcs/physical_props.f90:285-485): sums in
// the reference's loop order (k outer, i inner), the same operation order, no fused
// multiply-adds (this file is built with -ffp-contract=off), so that a run whose f equals
// the reference's writes the same bytes. Without f, the device moments are used and the
// columns that need phi (directional temperatures, entropy) are refused.
//
// Numbers are written with the edit descriptors of the reference's format statements, as
// gfortran writes them: Ew.d as [-]0.<d digits>E<sign><2 digits> (<sign><3 digits> past
// 99), right-justified; Iw right-justified; Aw right-justified when the text is shorter and
// cut to its leftmost w characters when longer (the property names are character(len=128)
// variables, blank-padded).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dvm_gpu.h"

namespace {

constexpr double kPiReference = 3.1459265358979323;  // utils/constants.f90:30 (sic)
constexpr double kPiExact = 3.14159265358979323846;
constexpr double kDoubleTol = 1.0e-13;                // utils/constants.f90:51

// property_names(1:27), input_output/visualization.f90:314-340
const char* const kPropertyNames[DVM_VIS_NPROP] = {
    "\"Density\"", "\"X-Velocity\"", "\"Y-Velocity\"", "\"Z-Velocity\"", "\"Speed\"",
    "\"Mach Number\"", "\"Trans. Temp.\"", "\"Rot. Temp.\"", "\"Vib. Temp.\"",
    "\"Total Temp.\"", "\"Temp. X\"", "\"Temp. Y\"", "\"Temp. Z\"", "\"Trans. Energy\"",
    "\"Rot. Energy\"", "\"Vib. Energy\"", "\"Total Energy\"", "\"Entropy\"",
    "\"Heat Flux X\"", "\"Heat Flux Y\"", "\"Heat Flux Z\"", "\"Rot DOF\"", "\"Vib DOF\"",
    "\"Rot. Temp Analytic\"", "\"Vib. Temp Analytic\"", "\"Trans. Temp Analytic\"",
    "\"Pressure\""};

// ---- edit descriptors ------------------------------------------------------------------
std::string ed_a(const std::string& s, int w) {
  if (static_cast<int>(s.size()) >= w) return s.substr(0, static_cast<size_t>(w));
  return std::string(static_cast<size_t>(w) - s.size(), ' ') + s;
}

// A character(len=128) variable holding s: blank-padded to 128 before Aw takes from it.
std::string ed_a128(const std::string& s, int w) {
  std::string v = s;
  v.resize(128, ' ');
  return ed_a(v, w);
}

std::string ed_i(long long n, int w) {
  const std::string s = std::to_string(n);
  if (static_cast<int>(s.size()) > w) return std::string(static_cast<size_t>(w), '*');
  return std::string(static_cast<size_t>(w) - s.size(), ' ') + s;
}

std::string ed_e(double x, int w, int d) {
  std::string body;
  if (std::isnan(x)) {
    body = "NaN";
  } else if (std::isinf(x)) {
    body = std::signbit(x) ? (w >= 9 ? "-Infinity" : "-Inf") : (w >= 8 ? "Infinity" : "Inf");
  } else {
    char buf[80];
    std::snprintf(buf, sizeof buf, "%.*e", d - 1, std::fabs(x));  // d significant digits
    std::string digits;
    const char* p = buf;
    digits += *p++;
    if (*p == '.') ++p;
    while (*p && *p != 'e') digits += *p++;
    const int e10 = (*p == 'e') ? std::atoi(p + 1) : 0;
    const int ex = (x == 0.0) ? 0 : e10 + 1;  // 0.ddd form
    std::string s = std::signbit(x) ? "-" : "";
    s += "0." + digits;
    char eb[16];
    const int ax = std::abs(ex);
    if (ax <= 99) std::snprintf(eb, sizeof eb, "E%c%02d", ex < 0 ? '-' : '+', ax);
    else if (ax <= 999) std::snprintf(eb, sizeof eb, "%c%03d", ex < 0 ? '-' : '+', ax);
    else return std::string(static_cast<size_t>(w), '*');
    s += eb;
    if (static_cast<int>(s.size()) > w) {  // the leading zero is optional
      const size_t z = s.find("0.");
      s.erase(z, 1);
    }
    body = s;
  }
  if (static_cast<int>(body.size()) > w) return std::string(static_cast<size_t>(w), '*');
  return std::string(static_cast<size_t>(w) - body.size(), ' ') + body;
}

// trim(adjustl(int2char(n))): the integer without blanks
std::string int2char(int n) { return std::to_string(n); }

bool cstr_ok(const char* s) { return s && s[0] && std::memchr(s, '\0', 128) != nullptr; }

// ---- the velocity grid and the properties of one cell ------------------------------------
struct Grid {
  int nx = 0, ny = 0, nz = 0;
  std::vector<double> x, y, z, bx, by, bz;
};

// compute_beta (grid/velocity_grid.f90:486-540)
void beta(const std::vector<double>& a, std::vector<double>& b) {
  const size_t n = a.size();
  b.assign(n, 0.0);
  b[0] = a[1] - a[0];
  b[n - 1] = a[n - 1] - a[n - 2];
  for (size_t i = 1; i + 1 < n; ++i) b[i] = (a[i + 1] - a[i]) / 2.0 + (a[i] - a[i - 1]) / 2.0;
}

bool make_grid(const dvm_vgrid* g, Grid& G) {
  if (!g || !g->x || !g->y || !g->z || g->nx < 2 || g->ny < 2 || g->nz < 2) return false;
  G.nx = g->nx; G.ny = g->ny; G.nz = g->nz;
  G.x.assign(g->x, g->x + g->nx);
  G.y.assign(g->y, g->y + g->ny);
  G.z.assign(g->z, g->z + g->nz);
  beta(G.x, G.bx);
  beta(G.y, G.by);
  beta(G.z, G.bz);
  return true;
}

// The fields of PropertiesType that the output reads, for one species (n = 1) and its
// mixture (physical_props.f90:41-69).
struct Cell {
  double dens = 0, x_vel = 0, y_vel = 0, z_vel = 0, avg_speed = 0;
  double species_tr_temp = 0, tr_temp = 0, temp = 0, species_temp = 0, pressure = 0;
  double tr_energy = 0, total_energy = 0;
  double mix_dens = 0, mix_x_vel = 0, mix_y_vel = 0, mix_z_vel = 0;
  double mix_tr_temp = 0, mix_temp = 0, mix_tr_energy = 0, mix_energy = 0;
};

// compute_temperature (physical_props.f90:1033-1087)
double temperature(const Grid& G, const double* f, double dens, double u, double v, double w,
                   double mass) {
  double t = 0.0;
  size_t l = 0;
  for (int k = 0; k < G.nz; ++k) {
    double czsq = G.z[k] - w;
    czsq = czsq * czsq;
    for (int j = 0; j < G.ny; ++j) {
      double cysq = G.y[j] - v;
      cysq = cysq * cysq;
      for (int i = 0; i < G.nx; ++i, ++l) {
        double cxsq = G.x[i] - u;
        cxsq = cxsq * cxsq;
        const double csq = cxsq + cysq + czsq;
        t = t + f[l] * csq;
      }
    }
  }
  return 2.0 * mass * t / (3.0 * dens);
}

// compute_overall_temperature (:1428-1457) with no internal degrees of freedom
double overall_temperature(double trans) {
  const double numerator = (3.0 * trans + 0.0 * 0.0 + 0.0 * 0.0);
  const double denominator = (3.0 + 0.0 + 0.0);
  return numerator / denominator;
}

// calculate_physical_properties (:285-485), one monatomic species, from f.
Cell cell_from_f(const Grid& G, const double* f, double mass) {
  Cell c;
  double dens = 0.0;
  const size_t nv = static_cast<size_t>(G.nx) * G.ny * G.nz;
  for (size_t l = 0; l < nv; ++l) dens = dens + f[l];  // compute_density
  c.dens = dens;
  if (dens == 0.0) return c;  // an empty cell: every field zero, mix_dens = dens
  double u = 0.0, v = 0.0, w = 0.0, as = 0.0;
  size_t l = 0;
  for (int k = 0; k < G.nz; ++k)
    for (int j = 0; j < G.ny; ++j)
      for (int i = 0; i < G.nx; ++i, ++l) u = u + f[l] * G.x[i];
  l = 0;
  for (int k = 0; k < G.nz; ++k)
    for (int j = 0; j < G.ny; ++j)
      for (int i = 0; i < G.nx; ++i, ++l) v = v + f[l] * G.y[j];
  l = 0;
  for (int k = 0; k < G.nz; ++k)
    for (int j = 0; j < G.ny; ++j)
      for (int i = 0; i < G.nx; ++i, ++l) w = w + f[l] * G.z[k];
  l = 0;
  for (int k = 0; k < G.nz; ++k) {
    const double czsq = G.z[k] * G.z[k];
    for (int j = 0; j < G.ny; ++j) {
      const double cysq = G.y[j] * G.y[j];
      for (int i = 0; i < G.nx; ++i, ++l) {
        const double cxsq = G.x[i] * G.x[i];
        as = as + f[l] * std::sqrt(cxsq + cysq + czsq);
      }
    }
  }
  c.x_vel = u / dens;
  c.y_vel = v / dens;
  c.z_vel = w / dens;
  c.avg_speed = as / dens;
  c.species_tr_temp = temperature(G, f, dens, c.x_vel, c.y_vel, c.z_vel, mass);
  c.tr_energy = 0.75 * c.dens * c.species_tr_temp;
  c.pressure = 0.5 * dens * c.species_tr_temp;
  // mixture of one species (compute_macro_density, compute_total_* :1300-1426)
  const double macro = 0.0 + mass * dens;
  c.mix_dens = 0.0 + dens;
  c.mix_x_vel = (0.0 + dens * mass * c.x_vel) / macro;
  c.mix_y_vel = (0.0 + dens * mass * c.y_vel) / macro;
  c.mix_z_vel = (0.0 + dens * mass * c.z_vel) / macro;
  c.tr_temp = temperature(G, f, dens, c.mix_x_vel, c.mix_y_vel, c.mix_z_vel, mass);
  c.mix_tr_temp = (0.0 + c.tr_temp * dens) / c.mix_dens;
  c.total_energy = 0.75 * c.dens * c.tr_temp + 0.0 + 0.0;
  c.temp = overall_temperature(c.tr_temp);
  c.species_temp = overall_temperature(c.species_tr_temp);
  c.mix_tr_energy = 0.75 * c.mix_dens * c.mix_tr_temp;
  c.mix_energy = c.mix_tr_energy + 0.0 + 0.0;
  c.mix_temp = (0.0 + c.temp * dens) / c.mix_dens;
  return c;
}

// The same fields from the device moments (no f): the species' own and the mixture's
// velocities and temperatures coincide for one species.
Cell cell_from_props(const double* P, double mass) {
  Cell c;
  c.dens = P[DVM_P_DENS];
  if (c.dens == 0.0) return c;
  c.x_vel = P[DVM_P_U]; c.y_vel = P[DVM_P_V]; c.z_vel = P[DVM_P_W];
  c.avg_speed = P[DVM_P_AVG_SPEED];
  c.species_tr_temp = P[DVM_P_TEMP];
  c.tr_temp = P[DVM_P_TEMP];
  c.tr_energy = 0.75 * c.dens * c.species_tr_temp;
  c.pressure = 0.5 * c.dens * c.species_tr_temp;
  const double macro = 0.0 + mass * c.dens;
  c.mix_dens = 0.0 + c.dens;
  c.mix_x_vel = (0.0 + c.dens * mass * c.x_vel) / macro;
  c.mix_y_vel = (0.0 + c.dens * mass * c.y_vel) / macro;
  c.mix_z_vel = (0.0 + c.dens * mass * c.z_vel) / macro;
  c.mix_tr_temp = (0.0 + c.tr_temp * c.dens) / c.mix_dens;
  c.total_energy = 0.75 * c.dens * c.tr_temp + 0.0 + 0.0;
  c.temp = overall_temperature(c.tr_temp);
  c.species_temp = overall_temperature(c.species_tr_temp);
  c.mix_tr_energy = 0.75 * c.mix_dens * c.mix_tr_temp;
  c.mix_energy = c.mix_tr_energy + 0.0 + 0.0;
  c.mix_temp = (0.0 + c.temp * c.dens) / c.mix_dens;
  return c;
}

enum { X_DIR = 1, Y_DIR = 2, Z_DIR = 3 };

// compute_directional_temperature (:1811-1869)
double directional_temperature(const Grid& G, const double* f, double dens, double vel, int dir,
                               double mass) {
  double t = 0.0;
  size_t l = 0;
  for (int k = 0; k < G.nz; ++k)
    for (int j = 0; j < G.ny; ++j)
      for (int i = 0; i < G.nx; ++i, ++l) {
        const double C = dir == X_DIR ? G.x[i] : (dir == Y_DIR ? G.y[j] : G.z[k]);
        const double csq = (C - vel) * (C - vel);
        t = t + f[l] * csq;
      }
  return (2.0 / 3.0) * mass * t / dens;
}

// compute_entropy (:1871-1912), C = 1
double entropy(const Grid& G, const double* f) {
  double s = 0.0;
  const size_t nv = static_cast<size_t>(G.nx) * G.ny * G.nz;
  for (size_t l = 0; l < nv; ++l) {
    if (f[l] == 0.0) continue;
    s = s - std::fabs(f[l]) * std::log(1.0 * std::fabs(f[l]));
  }
  return s;
}

// compute_heat_flux (:1914-1986)
double heat_flux(const Grid& G, const double* f, double u, double v, double w, double dens,
                 int dir, double mass) {
  if (dens == 0.0) return 0.0;
  double q = 0.0;
  size_t l = 0;
  for (int k = 0; k < G.nz; ++k) {
    const double z = G.z[k];
    const double czsq = (z - w) * (z - w);
    for (int j = 0; j < G.ny; ++j) {
      const double y = G.y[j];
      const double cysq = (y - v) * (y - v);
      for (int i = 0; i < G.nx; ++i, ++l) {
        const double x = G.x[i];
        const double cxsq = (x - u) * (x - u);
        const double csq = cxsq + cysq + czsq;
        const double c = dir == X_DIR ? (x - u) : (dir == Y_DIR ? (y - v) : (z - w));
        q = q + c * csq * f[l];
      }
    }
  }
  return q * (0.5 * mass);
}

// compute_viscous_stress (:1988-2071), direction 11, 22, 33, 12, 13 or 23
double viscous_stress(const Grid& G, const double* f, int dir, double u, double v, double w,
                      double pressure, double mass) {
  double tau = 0.0;
  size_t l = 0;
  for (int k = 0; k < G.nz; ++k)
    for (int j = 0; j < G.ny; ++j)
      for (int i = 0; i < G.nx; ++i, ++l) {
        const double cx = G.x[i] - u, cy = G.y[j] - v, cz = G.z[k] - w;
        double v1, v2;
        switch (dir) {
          case 11: v1 = cx; v2 = cx; break;
          case 22: v1 = cy; v2 = cy; break;
          case 33: v1 = cz; v2 = cz; break;
          case 12: v1 = cx; v2 = cy; break;
          case 13: v1 = cx; v2 = cz; break;
          default: v1 = cy; v2 = cz; break;
        }
        tau = tau - v1 * v2 * f[l];
      }
  return (dir == 11 || dir == 22 || dir == 33) ? pressure + mass * tau : mass * tau;
}

// compute_moment (:2073-2128): the moment of order d of |c - u| normalised by its
// Maxwell-Boltzmann value, (d+1)!! T^(1.5+d) 2^(-d/2)
double moment(const Grid& G, const double* f, int flag, double dens, double u, double v,
              double w, double temp, double mass) {
  const double d = static_cast<double>(flag);
  double nfact = 1.0;
  for (int in = 1;; in -= 2) {
    const double change = static_cast<double>(flag + in);
    if (flag + in >= 1) nfact = nfact * change;
    else break;
  }
  const double mom_MB = nfact * std::pow(temp, 1.5 + d) * std::pow(2.0, -0.5 * d);
  double m = 0.0;
  size_t l = 0;
  for (int k = 0; k < G.nz; ++k) {
    double czsq = G.z[k] - w;
    czsq = czsq * czsq;
    for (int j = 0; j < G.ny; ++j) {
      double cysq = G.y[j] - v;
      cysq = cysq * cysq;
      for (int i = 0; i < G.nx; ++i, ++l) {
        double cxsq = G.x[i] - u;
        cxsq = cxsq * cxsq;
        const double C = std::sqrt(cxsq + cysq + czsq);
        m = m + std::pow(C, d) * f[l];
      }
    }
  }
  return std::pow(mass, 0.5 * d) * m / (dens * mom_MB);
}

double stress_from_props(const double* P, int dir) {
  switch (dir) {
    case 11: return P[DVM_P_TXX];
    case 22: return P[DVM_P_TYY];
    case 33: return P[DVM_P_TZZ];
    case 12: return P[DVM_P_TXY];
    case 13: return P[DVM_P_TXZ];
    default: return P[DVM_P_TYZ];
  }
}

bool valid_stress(int d) {
  return d == 11 || d == 22 || d == 33 || d == 12 || d == 13 || d == 23;
}

int check_vis(const dvm_vis* v) {
  if (!v || v->nx_space < 1 || v->ny_space < 1 || v->write_stress < 0 || v->write_stress > 6 ||
      !(v->mass > 0.0))
    return DVM_ERR_PARAM;
  for (int i = 0; i < v->write_stress; ++i)
    if (!valid_stress(v->stress_directions[i])) return DVM_ERR_PARAM;
  if (v->write_moment < 0 || v->write_moment > 6) return DVM_ERR_PARAM;
  return DVM_OK;
}

// calculate_specific_heat_ratio and calculate_molecular_mass (conditions/shock_conditions.f90:
// 222-314) for one monatomic species, from the right wall's density
void gas_constants(const dvm_vis* v, double& gamma, double& mol_mass) {
  const double dens = v->right_wall_dens, mass = v->mass;
  const double dof = 0.0 + 3.0 + 0.0;
  double cp_mix = 0.0, total_mass = 0.0;
  total_mass = total_mass + mass * dens;
  cp_mix = cp_mix + mass * dens * (dof * 0.5 + 1.0);
  cp_mix = cp_mix / total_mass;
  gamma = cp_mix / (cp_mix - 1.0);
  double tot_dens = 0.0;
  mol_mass = 0.0;
  tot_dens = tot_dens + dens;
  mol_mass = mol_mass + dens * mass;
  mol_mass = mol_mass / tot_dens;
}

void write_zone_header_line(FILE* fp, const dvm_vis* v) {
  if (v->nx_space == 1) {
    const int freq = v->properties_dump_freq > 0 ? v->properties_dump_freq : 1;
    const int pt = (v->end_time % freq == 0) ? v->end_time / freq + 1 : v->end_time / freq + 2;
    std::fprintf(fp, "zone i=%s\n", ed_i(pt, 4).c_str());
  }
}

std::string df_path(const dvm_vis* v, int loc) {
  return std::string(v->df_filename) + "_1_" + int2char(v->x_locations[loc]) + "_" +
         int2char(v->y_locations[loc]) + ".dat";
}

}  // namespace

extern "C" int dvm_vis_write_headers(const dvm_vis* v) {
  int st = check_vis(v);
  if (st) return st;
  if (v->enable_properties) {
    if (!cstr_ok(v->properties_filename)) return DVM_ERR_PARAM;
    const std::string base(v->properties_filename);
    // the mixture file: names through (a3,a14)
    FILE* fp = std::fopen((base + ".dat").c_str(), "w");
    if (!fp) return DVM_ERR_IO;
    std::fprintf(fp, "title = \"Macroscopic Properties\"\n");
    std::fprintf(fp, "variables = \"Time\", \"x-Location\", \"y-Location\"");
    for (int i = 0; i < DVM_VIS_NPROP; ++i)
      if (v->properties_to_output[i])
        std::fprintf(fp, "%s%s", ed_a(", ", 3).c_str(), ed_a128(kPropertyNames[i], 14).c_str());
    for (int i = 0; i < v->write_stress; ++i)
      std::fprintf(fp, ", \"Tau %s\"", ed_i(v->stress_directions[i], 2).c_str());
    for (int i = 0; i < v->write_moment; ++i)
      std::fprintf(fp, ", \"Moment %s\"", ed_i(v->moment_numbers[i], 2).c_str());
    std::fprintf(fp, " \n");
    write_zone_header_line(fp, v);
    if (std::fclose(fp)) return DVM_ERR_IO;
    // the species file: names through (a2,a), trimmed
    fp = std::fopen((base + "_1.dat").c_str(), "w");
    if (!fp) return DVM_ERR_IO;
    std::fprintf(fp, "title = \"Macroscopic Properties\"\n");
    std::fprintf(fp, "variables = \"Time\", \"x-Location\", \"y-Location\"");
    for (int i = 0; i < DVM_VIS_NPROP; ++i)
      if (v->properties_to_output[i]) std::fprintf(fp, ", %s", kPropertyNames[i]);
    for (int i = 0; i < v->write_stress; ++i)
      std::fprintf(fp, ", \"Tau %s\"", ed_i(v->stress_directions[i], 2).c_str());
    for (int i = 0; i < v->write_moment; ++i)
      std::fprintf(fp, ", \"Moment %s\"", ed_i(v->moment_numbers[i], 2).c_str());
    std::fprintf(fp, " \n");
    write_zone_header_line(fp, v);
    if (std::fclose(fp)) return DVM_ERR_IO;
  }
  const bool df = v->enable_vel_df || v->enable_rot_df || v->enable_vib_df;
  if (df) {
    if (!cstr_ok(v->df_filename) || v->num_locations < 1 || v->num_locations > 16 ||
        v->df_dimension < DVM_VIS_DF_1D || v->df_dimension > DVM_VIS_DF_3D ||
        v->rot_levels < 0 || v->vib_levels < 0)
      return DVM_ERR_PARAM;
    for (int loc = 0; loc < v->num_locations; ++loc) {
      FILE* fp = std::fopen(df_path(v, loc).c_str(), "w");
      if (!fp) return DVM_ERR_IO;
      std::fprintf(fp, "title = \"Distribution Function\"\n");
      if (v->df_dimension == DVM_VIS_DF_1D)
        std::fprintf(fp, "variables = \"X-Velocity\", \"Beta3\", \"Time\"");
      else if (v->df_dimension == DVM_VIS_DF_2D)
        std::fprintf(fp, "variables = \"X-Velocity\", \"Y-Velocity\", \"Beta3\", \"Time\"");
      else
        std::fprintf(fp, "variables = \"X-Velocity\", \"Y-Velocity\", \"Z-Velocity\", "
                         "\"Beta3\", \"Time\"");
      if (v->enable_vel_df) std::fprintf(fp, ", \"Vel DistFunc\", \"Deviation\"");
      if (v->enable_rot_df) {
        for (int l = 1; l <= v->rot_levels; ++l) std::fprintf(fp, ", \"Rot %s\"", ed_i(l, 3).c_str());
        std::fprintf(fp, ", \"Rot Energy\"");
      }
      if (v->enable_vib_df) {
        for (int l = 1; l <= v->vib_levels; ++l) std::fprintf(fp, ", \"Vib %s\"", ed_i(l, 3).c_str());
        std::fprintf(fp, ", \"Vib Energy\"");
      }
      std::fprintf(fp, " \n");
      if (std::fclose(fp)) return DVM_ERR_IO;
    }
  }
  return DVM_OK;
}

extern "C" int dvm_vis_write_properties(const dvm_vis* v, double time, const double* props,
                                        const double* f, const dvm_vgrid* grid) {
  int st = check_vis(v);
  if (st) return st;
  if (!v->enable_properties) return DVM_OK;
  if (!cstr_ok(v->properties_filename) || (!props && !f)) return DVM_ERR_PARAM;
  const int* out = v->properties_to_output;
  Grid G;
  const bool need_grid = f != nullptr;
  if (need_grid && !make_grid(grid, G)) return DVM_ERR_PARAM;
  // columns formed from phi need f
  if (!f && (out[10] || out[11] || out[12] || out[17] || v->write_moment > 0))
    return DVM_ERR_PARAM;
  const int ncells = v->nx_space * v->ny_space;
  const size_t nv = need_grid ? static_cast<size_t>(G.nx) * G.ny * G.nz : 0;
  double gamma = 0.0, mol_mass = 0.0;
  gas_constants(v, gamma, mol_mass);
  std::vector<double> total(static_cast<size_t>(ncells) * DVM_VIS_NPROP, 0.0);
  std::vector<double> species(static_cast<size_t>(ncells) * DVM_VIS_NPROP, 0.0);
  std::vector<double> tstress(static_cast<size_t>(ncells) * 6, 0.0);
  std::vector<double> smom(static_cast<size_t>(ncells) * 6, 0.0);
  double coeff = 1.596;  // get_data_to_output keeps multiplying one coefficient
  for (int nx = 0; nx < v->nx_space; ++nx)
    for (int ny = 0; ny < v->ny_space; ++ny) {
      const int cell = nx + v->nx_space * ny;
      const double* fc = f ? f + static_cast<size_t>(cell) * nv : nullptr;
      const double* P = props ? props + static_cast<size_t>(cell) * DVM_NPROP : nullptr;
      const Cell c = fc ? cell_from_f(G, fc, v->mass) : cell_from_props(P, v->mass);
      double* T = total.data() + static_cast<size_t>(cell) * DVM_VIS_NPROP;
      double* S = species.data() + static_cast<size_t>(cell) * DVM_VIS_NPROP;
      if (out[0]) { S[0] = c.dens; T[0] = c.mix_dens; }
      if (out[1]) { S[1] = c.x_vel; T[1] = c.mix_x_vel; }
      if (out[2]) { S[2] = c.y_vel; T[2] = c.mix_y_vel; }
      if (out[3]) { S[3] = c.z_vel; T[3] = c.mix_z_vel; }
      if (out[4]) {  // compute_speed (:1779-1790)
        S[4] = std::sqrt(c.x_vel * c.x_vel + c.y_vel * c.y_vel + c.z_vel * c.z_vel);
        T[4] = std::sqrt(c.mix_x_vel * c.mix_x_vel + c.mix_y_vel * c.mix_y_vel +
                         c.mix_z_vel * c.mix_z_vel);
      }
      if (out[5]) {
        S[5] = c.x_vel / std::sqrt(0.5 * gamma * c.tr_temp / mol_mass);
        T[5] = c.mix_x_vel / std::sqrt(0.5 * gamma * c.mix_tr_temp / mol_mass);
      }
      if (out[6]) { S[6] = c.species_tr_temp; T[6] = c.mix_tr_temp; }
      // 8, 9: no rotational or vibrational modes: zero temperatures
      if (out[9]) { S[9] = c.temp; T[9] = c.mix_temp; }
      if (out[10]) S[10] = directional_temperature(G, fc, c.dens, c.x_vel, X_DIR, v->mass);
      if (out[11]) S[11] = directional_temperature(G, fc, c.dens, c.y_vel, Y_DIR, v->mass);
      if (out[12]) S[12] = directional_temperature(G, fc, c.dens, c.z_vel, Z_DIR, v->mass);
      if (out[13]) { S[13] = c.tr_energy; T[13] = c.mix_tr_energy; }
      if (out[16]) { S[16] = c.total_energy; T[16] = c.mix_energy; }
      if (out[17]) { S[17] = entropy(G, fc); T[17] = 0.0 + S[17]; }
      for (int d = 0; d < 3; ++d)
        if (out[18 + d]) {
          S[18 + d] = fc ? heat_flux(G, fc, c.x_vel, c.y_vel, c.z_vel, c.dens, X_DIR + d, v->mass)
                         : P[DVM_P_QX + d];
          T[18 + d] = 0.0 + S[18 + d];
        }
      // 22, 23: degrees of freedom, zero
      const bool t0 = std::fabs(time) < kDoubleTol;
      const double trn_dof = 5.0 - 2.0 * v->omega;
      if (out[23]) {  // analytic rotational relaxation
        if (t0) {
          S[23] = 0.0;
        } else {
          const double T_eq = 4.0 * (c.tr_energy + 0.0) / (c.dens * (3.0 + 0.0));
          coeff = coeff * (trn_dof + 0.0) / trn_dof;
          const double coll_freq = coeff * std::pow(c.species_tr_temp, 1.0 - v->omega);
          S[23] = T_eq - (T_eq - v->right_wall_temp_rot) * std::exp(-coll_freq * time / v->cZr);
        }
      }
      if (out[24]) {
        if (t0) {
          S[24] = 0.0;
        } else {
          const double T_eq = 4.0 * (c.tr_energy + 0.0) / (c.dens * (3.0 + 0.0));
          coeff = coeff * (trn_dof + 0.0) / trn_dof;
          const double coll_freq = coeff * std::pow(c.species_tr_temp, 1.0 - v->omega);
          S[24] = T_eq - (T_eq - v->right_wall_temp_vib) * std::exp(-coll_freq * time / v->cZv);
        }
      }
      if (out[25])
        S[25] = t0 ? c.tr_temp
                   : (4.0 / 3.0) * (c.total_energy - (0.0 / 4.0) * S[23] - (0.0 / 4.0) * S[24]);
      if (out[26]) {
        S[26] = 0.5 * c.dens * c.tr_temp;
        T[26] = 0.5 * c.mix_dens * c.mix_tr_temp;
      }
      for (int i = 0; i < v->write_stress; ++i) {
        const int dir = v->stress_directions[i];
        const double tau = fc ? viscous_stress(G, fc, dir, c.x_vel, c.y_vel, c.z_vel, c.pressure,
                                               v->mass)
                              : stress_from_props(P, dir);
        tstress[static_cast<size_t>(cell) * 6 + i] = 0.0 + tau;
      }
      for (int i = 0; i < v->write_moment; ++i)
        smom[static_cast<size_t>(cell) * 6 + i] =
            moment(G, fc, v->moment_numbers[i], c.dens, c.x_vel, c.y_vel, c.z_vel, c.tr_temp,
                   v->mass);
    }
  const std::string base(v->properties_filename);
  for (int file = 0; file < 2; ++file) {
    FILE* fp = std::fopen((base + (file == 0 ? ".dat" : "_1.dat")).c_str(), "a");
    if (!fp) return DVM_ERR_IO;
    // the mixture file opens a zone for any multi-cell run, the species file only when
    // nx_space > 1; their locations start at half a cell and at zero
    if (file == 0 ? (v->nx_space > 1 || v->ny_space > 1) : v->nx_space > 1)
      std::fprintf(fp, "zone i=%s\n", ed_i(static_cast<long long>(ncells), 5).c_str());
    const std::vector<double>& D = file == 0 ? total : species;
    double x_location = file == 0 ? 0.5 * v->dx : 0.0;
    for (int nx = 0; nx < v->nx_space; ++nx) {
      double y_location = file == 0 ? 0.5 * v->dy : 0.0;
      for (int ny = 0; ny < v->ny_space; ++ny) {
        const int cell = nx + v->nx_space * ny;
        std::string row = ed_e(time, 24, 15) + ed_e(x_location, 24, 15) + ed_e(y_location, 24, 15);
        for (int p = 0; p < DVM_VIS_NPROP; ++p)
          if (out[p]) row += ed_e(D[static_cast<size_t>(cell) * DVM_VIS_NPROP + p], 24, 16);
        for (int i = 0; i < v->write_stress; ++i)
          row += ed_e(tstress[static_cast<size_t>(cell) * 6 + i], 24, 16);
        for (int i = 0; i < v->write_moment; ++i)  // total_moments are zero
          row += ed_e(file == 0 ? 0.0 : smom[static_cast<size_t>(cell) * 6 + i], 24, 16);
        std::fprintf(fp, "%s \n", row.c_str());
        y_location = y_location + v->dy;
      }
      x_location = x_location + v->dx;
    }
    if (std::fclose(fp)) return DVM_ERR_IO;
  }
  return DVM_OK;
}

extern "C" int dvm_vis_write_df(const dvm_vis* v, double time, const double* f,
                                const dvm_vgrid* grid) {
  int st = check_vis(v);
  if (st) return st;
  const bool df = v->enable_vel_df || v->enable_rot_df || v->enable_vib_df;
  if (!df) return DVM_OK;
  if (!f || !cstr_ok(v->df_filename) || v->num_locations < 1 || v->num_locations > 16 ||
      v->df_dimension < DVM_VIS_DF_1D || v->df_dimension > DVM_VIS_DF_3D)
    return DVM_ERR_PARAM;
  Grid G;
  if (!make_grid(grid, G)) return DVM_ERR_PARAM;
  const size_t nv = static_cast<size_t>(G.nx) * G.ny * G.nz;
  const double pi = v->pi_mode == DVM_PI_EXACT ? kPiExact : kPiReference;
  // i_zero, j_zero: the first node within double_tol of zero (write_df :995-1010); k_zero:
  // find_zero_point's zero node (grid/velocity_grid.f90:653-689), the last node <= 0
  int i_zero = -1, j_zero = -1, k_zero = -1;
  for (int i = 0; i < G.nx && i_zero < 0; ++i)
    if (std::fabs(G.x[i]) < kDoubleTol) i_zero = i;
  for (int j = 0; j < G.ny && j_zero < 0; ++j)
    if (std::fabs(G.y[j]) < kDoubleTol) j_zero = j;
  if (!(G.z[0] > 0.0)) {
    k_zero = G.nz - 1;
    for (int k = 1; k < G.nz; ++k)
      if (G.z[k] > 0.0) { k_zero = k - 1; break; }
  }
  if ((v->df_dimension == DVM_VIS_DF_1D && (j_zero < 0 || k_zero < 0)) ||
      (v->df_dimension == DVM_VIS_DF_2D && k_zero < 0))
    return DVM_ERR_PARAM;  // the reference leaves the plane index undefined there
  (void)i_zero;
  for (int loc = 0; loc < v->num_locations; ++loc) {
    const int cx = v->x_locations[loc] - 1, cy = v->y_locations[loc] - 1;
    if (cx < 0 || cx >= v->nx_space || cy < 0 || cy >= v->ny_space) return DVM_ERR_PARAM;
    const int cell = cx + v->nx_space * cy;
    const double* fc = f + static_cast<size_t>(cell) * nv;
    // the cell's properties as the reference holds them: formed from its phi
    const Cell use = cell_from_f(G, fc, v->mass);
    const double mass = v->mass, dens = use.dens, u = use.x_vel, vv = use.y_vel, w = use.z_vel;
    const double temp = use.mix_temp;
    const double coeff = dens > 0.0 ? dens * std::sqrt(mass * mass * mass) /
                                          std::sqrt(pi * pi * pi * temp * temp * temp)
                                    : 0.0;
    auto maxwell = [&](double x, double y, double z) {  // compute_maxwellian
      double cxsq = (x - u);
      cxsq = cxsq * cxsq;
      double cysq = (y - vv);
      cysq = cysq * cysq;
      double czsq = (z - w);
      czsq = czsq * czsq;
      const double csq = cxsq + cysq + czsq;
      return coeff * std::exp(-csq * mass / temp);
    };
    FILE* fp = std::fopen(df_path(v, loc).c_str(), "a");
    if (!fp) return DVM_ERR_IO;
    auto tail = [&](std::string& row, size_t l, double df_eq) {
      if (v->enable_vel_df) row += ed_e(fc[l], 24, 16) + ed_e(fc[l] - df_eq, 24, 16);
      if (v->enable_rot_df) {
        for (int q = 0; q < v->rot_levels; ++q) row += ed_e(0.0, 24, 16);
        row += ed_e(0.0, 24, 16);
      }
      if (v->enable_vib_df) {
        for (int q = 0; q < v->vib_levels; ++q) row += ed_e(0.0, 24, 16);
        row += ed_e(0.0, 24, 16);
      }
      std::fprintf(fp, "%s \n", row.c_str());
    };
    if (v->df_dimension == DVM_VIS_DF_1D) {
      std::fprintf(fp, "zone i=%s\n", ed_i(G.nx, 4).c_str());
      const int j = j_zero, k = k_zero;
      for (int i = 0; i < G.nx; ++i) {
        const double beta3 = G.bx[i] * G.by[j] * G.bz[k];
        double df_eq = temp > 0.0 ? maxwell(G.x[i], 0.0, 0.0) : 0.0;
        df_eq = df_eq * beta3;
        std::string row = ed_e(G.x[i], 24, 16) + ed_e(beta3, 24, 16) + ed_e(time, 24, 16);
        tail(row, static_cast<size_t>(i) + static_cast<size_t>(G.nx) * (j + static_cast<size_t>(G.ny) * k), df_eq);
      }
    } else if (v->df_dimension == DVM_VIS_DF_2D) {
      std::fprintf(fp, "zone i=%s, j=%s\n", ed_i(G.nx, 3).c_str(), ed_i(G.ny, 3).c_str());
      const int k = k_zero;
      for (int j = 0; j < G.ny; ++j)
        for (int i = 0; i < G.nx; ++i) {
          const double beta3 = G.bx[i] * G.by[j] * G.bz[k];
          double df_eq = temp > 0.0 ? maxwell(G.x[i], G.y[j], 0.0) : 0.0;
          df_eq = df_eq * beta3;
          std::string row = ed_e(G.x[i], 24, 16) + ed_e(G.y[j], 24, 16) + ed_e(beta3, 24, 16) +
                            ed_e(time, 24, 16);
          tail(row, static_cast<size_t>(i) + static_cast<size_t>(G.nx) * (j + static_cast<size_t>(G.ny) * k), df_eq);
        }
    } else {
      std::fprintf(fp, "zone i=%s%s%s%s%s\n", ed_i(G.nx, 4).c_str(), ed_a(", j=", 9).c_str(),
                   ed_i(G.ny, 4).c_str(), ed_a(", k=", 9).c_str(), ed_i(G.nz, 4).c_str());
      for (int k = 0; k < G.nz; ++k)
        for (int j = 0; j < G.ny; ++j)
          for (int i = 0; i < G.nx; ++i) {
            const double beta3 = G.bx[i] * G.by[j] * G.bz[k];
            double df_eq = temp > 0.0 ? maxwell(G.x[i], G.y[j], G.z[k]) : 0.0;
            df_eq = df_eq * beta3;
            std::string row = ed_e(G.x[i], 24, 16) + ed_e(G.y[j], 24, 16) +
                              ed_e(G.z[k], 24, 16) + ed_e(beta3, 24, 16) + ed_e(time, 24, 16);
            tail(row, static_cast<size_t>(i) + static_cast<size_t>(G.nx) * (j + static_cast<size_t>(G.ny) * k), df_eq);
          }
    }
    if (std::fclose(fp)) return DVM_ERR_IO;
  }
  return DVM_OK;
}

// The edit descriptors alone, so that they can be checked against hand-written Fortran
// output without writing files.
extern "C" int dvm_vis_format_e(double x, int w, int d, char* out, int out_len) {
  if (!out || out_len < w + 1 || w < 1 || w > 64 || d < 1 || d > 40) return DVM_ERR_PARAM;
  const std::string s = ed_e(x, w, d);
  std::memcpy(out, s.c_str(), s.size() + 1);
  return DVM_OK;
}
