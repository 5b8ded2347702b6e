// dvm_host.cpp -- C++ host of the GPU time step: the reference driver's program flow
// (main.f90:25-38: initialize_solver, solve, destroy_solver in solver/dvm_solver.f90)
// running through the C ABI of include/dvm_gpu.h.
//
//   dvm_host <input deck> [--check] [--steps N] [--dump-f FILE] [--dump-props FILE]
//            [--restart-in FILE] [--restart-out FILE]
//
// The deck is the reference's `key = value` format (input_output/read_input_2D.f90:75-777;
// e.g. trunk/bin/velocity_refined.inp): [sections] and `#` comments are skipped, values may
// be quoted and may use Fortran exponents (1.0d0); a key holding several entries (one per
// species or zone, '11 11') gives its first, as the reference's per-species reads do for
// species 1. Keys read: Kn, species_codes, csection_method, csection_coeff, delta_x,
// delta_y, nx_space, ny_space, deltat, ntstep, num_points_{x,y,z}, {x,y,z}v_{min,max},
// InitC, InitDF, spatial_middle, dens_init, {x,y,z}_vel_init, tr_temp_init,
// {x,y,z}_delta_loc, {dens,x_vel,y_vel,z_vel,tr_temp}_{LW,RW,BW,TW}, {L,R,B,T}WallBC,
// acc_coeff, iColl, cdf_tolerance, NRepl, ColnRMS, iConv, display_freq, and the output keys
// of the [vis] section (enable_properties_vis, properties_vis_filename,
// properties_vis_dump_freq, write_* of each property, write_stress, stress_directions,
// write_moment, moment_numbers, enable_{vel,rot,vib}_df_vis, df_vis_filename,
// df_vis_dump_freq, num_output_locations, {x,y}_output_locations, df_output_dimension,
// num_rot_levels, num_vib_levels). Decks of the earlier GRVY reader name the cell count
// nspace; it is read as nx_space when nx_space is absent, and num_zones > 1 (per-zone
// velocity grids) is refused. Keys this build adds: geometry, samples_per_step, seed,
// pi_mode, and for the initial states of the benchmark configurations InitC = 6 (two
// drifting Maxwellians: bimodal_T_ratio, bimodal_drift) and InitC = 7 (Rankine-Hugoniot
// shock joined by a tanh profile: mach_number, shock_width).
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "dvm_gpu.h"

namespace {

constexpr double kPiReference = 3.1459265358979323;  // utils/constants.f90:30 (sic)
constexpr double kPiExact = 3.14159265358979323846;

struct Deck {
  std::map<std::string, std::string> kv;

  static std::string trim(const std::string& s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace(static_cast<unsigned char>(s[a]))) ++a;
    while (b > a && std::isspace(static_cast<unsigned char>(s[b - 1]))) --b;
    return s.substr(a, b - a);
  }

  bool load(const char* path) {
    std::ifstream in(path);
    if (!in) return false;
    std::string line;
    while (std::getline(in, line)) {
      const size_t hash = line.find('#');
      if (hash != std::string::npos) line = line.substr(0, hash);
      line = trim(line);
      if (line.empty() || line[0] == '[') continue;
      const size_t eq = line.find('=');
      if (eq == std::string::npos) continue;
      std::string key = trim(line.substr(0, eq)), val = trim(line.substr(eq + 1));
      val.erase(std::remove(val.begin(), val.end(), '\''), val.end());
      kv[key] = trim(val);
    }
    return true;
  }
  bool has(const std::string& k) const { return kv.count(k) > 0; }
  std::string str(const std::string& k, const std::string& def) const {
    auto it = kv.find(k);
    if (it == kv.end()) return def;
    std::istringstream ss(it->second);  // vector values: first entry
    std::string first;
    ss >> first;
    return first;
  }
  double num(const std::string& k, double def) const {
    std::string v = str(k, "");
    if (v.empty()) return def;
    for (char& ch : v)
      if (ch == 'd' || ch == 'D') ch = 'e';  // Fortran double exponent
    return std::strtod(v.c_str(), nullptr);
  }
  long long integer(const std::string& k, long long def) const {
    std::string v = str(k, "");
    return v.empty() ? def : std::strtoll(v.c_str(), nullptr, 10);
  }
  // every entry of a vector key (x_output_locations = '1 4')
  std::vector<long long> integers(const std::string& k) const {
    std::vector<long long> out;
    auto it = kv.find(k);
    if (it == kv.end()) return out;
    std::istringstream ss(it->second);
    std::string tok;
    while (ss >> tok) out.push_back(std::strtoll(tok.c_str(), nullptr, 10));
    return out;
  }
};

// gamma_calculator (utils/math_utils.f90:79-135): Lanczos, g = 7, the nine published
// coefficients, with the pi the run uses.
double gamma_fn(double x, double pi) {
  static const double c[9] = {0.99999999999980993, 676.5203681218851, -1259.1392167224028,
                              771.32342877765313, -176.61502916214059, 12.507343278686905,
                              -0.13857109526572012, 9.9843695780195716e-6,
                              1.5056327351493116e-7};
  if (x < 0.5) return pi / (std::sin(pi * x) * gamma_fn(1.0 - x, pi));
  x = x - 1.0;
  double y = c[0];
  for (int i = 1; i <= 8; ++i) y = y + c[i] / (x + static_cast<double>(i));
  const double z = x + 7.0 + 0.5;
  return std::sqrt(2.0 * pi) * std::pow(z, x + 0.5) * std::exp(-z) * y;
}

struct Species {
  double diam, mass, omega, alpha;
};

bool species_data(const std::string& code, Species& s) {
  // input_output/species_data.f90:255-304 (single-precision literals in the reference)
  if (code == "He") s = {2.33e-10f, 6.65e-27f, 0.66, 1.31};
  else if (code == "Ne") s = {2.77e-10f, 33.5e-27f, 0.66, 1.31};
  else if (code == "Ar") s = {4.17e-10f, 66.3e-27f, 0.81, 1.40};
  else if (code == "Xe") s = {5.74e-10f, 218.e-27f, 0.85, 1.44};
  else return false;
  return true;
}

class Host {
 public:
  dvm_params p{};
  std::vector<double> x, y, z;
  int ncells = 0, nv = 0;
  long long ntstep = 0;
  int display_freq = 50;
  std::vector<double> f;
  dvm_ctx* ctx = nullptr;

  // read_input_grvy + set_molecule_constants + create_velocity_grid (host side)
  bool read_input(const Deck& d, std::string& err) {
    std::memset(&p, 0, sizeof(p));
    if (d.integer("num_zones", 1) > 1) {
      err = "num_zones = " + d.str("num_zones", "") +
            ": per-zone velocity grids are not supported (one grid for every cell)";
      return false;
    }
    // the earlier reader's name for the cell count
    p.nx_space = static_cast<int>(d.has("nx_space") ? d.integer("nx_space", 1)
                                                    : d.integer("nspace", 1));
    p.ny_space = static_cast<int>(d.integer("ny_space", 1));
    const int geo_default = (p.nx_space == 1 && p.ny_space == 1) ? DVM_GEOM_0D
                            : (p.ny_space == 1 ? DVM_GEOM_1D : DVM_GEOM_2D);
    p.geometry = static_cast<int>(d.integer("geometry", geo_default));
    p.dx = d.num("delta_x", 1.0);
    p.dy = d.num("delta_y", 1.0);
    p.dt = d.num("deltat", 0.01);
    p.Kn = d.num("Kn", 1.0);
    p.pi_mode = static_cast<int>(d.integer("pi_mode", DVM_PI_REFERENCE));
    const double pi = p.pi_mode == DVM_PI_EXACT ? kPiExact : kPiReference;
    Species sp;
    const std::string code = d.str("species_codes", "Ar");
    if (!species_data(code, sp)) { err = "unsupported species " + code; return false; }
    // single species = reference species: mass and diameter scale to 1
    const double mass = 1.0, diam = 1.0;
    const int cs_method = static_cast<int>(d.integer("csection_method", 1));
    double omega = sp.omega, alpha = sp.alpha;
    if (cs_method == 1) { omega = 0.5; alpha = 1.0; }
    else if (cs_method == 2) { omega = 1.0; alpha = 1.0; }
    else if (cs_method == 3) { alpha = 1.0; }
    p.mass = mass; p.omega = omega; p.alpha = alpha;
    // calculate_cross_section (solver/scaling.f90:163-201), like-species pair
    const double m_red = mass * mass / (mass + mass);
    const double sigma_vhs = 0.25 * (diam + diam) * (diam + diam);
    const int cs_coeff = static_cast<int>(d.integer("csection_coeff", 2));
    if (cs_coeff == 1) p.sigma = sigma_vhs;
    else if (cs_coeff == 2) p.sigma = sigma_vhs * std::pow(m_red, 0.5 - omega) / gamma_fn(2.5 - omega, pi);
    else { err = "csection_coeff " + std::to_string(cs_coeff) + " not supported"; return false; }
    p.coll_method = static_cast<int>(d.integer("iColl", DVM_COLL_VR));
    p.conv_method = static_cast<int>(d.integer("iConv", DVM_CONV_NONE));
    p.num_repl = static_cast<int>(d.integer("NRepl", 1));
    p.coln_rms = d.num("ColnRMS", 0.001);
    p.cdf_tolerance = d.num("cdf_tolerance", 0.01);
    p.acc_coeff = d.num("acc_coeff", 1.0);
    if (d.has("samples_per_step")) {
      p.samples_mode = DVM_SAMPLES_FIXED;
      p.samples_per_step = d.integer("samples_per_step", 0);
    }
    p.seed = static_cast<uint64_t>(d.integer("seed", 0));
    const char* wn[4] = {"LW", "RW", "BW", "TW"};
    const char* bn[4] = {"LWallBC", "RWallBC", "BWallBC", "TWallBC"};
    for (int w = 0; w < 4; ++w) {
      p.bc[w] = static_cast<int>(d.integer(bn[w], 1));
      p.wall[w][DVM_WP_DENS] = d.num(std::string("dens_") + wn[w], 1.0);
      p.wall[w][DVM_WP_U] = d.num(std::string("x_vel_") + wn[w], 0.0);
      p.wall[w][DVM_WP_V] = d.num(std::string("y_vel_") + wn[w], 0.0);
      p.wall[w][DVM_WP_W] = d.num(std::string("z_vel_") + wn[w], 0.0);
      p.wall[w][DVM_WP_TEMP] = d.num(std::string("tr_temp_") + wn[w], 1.0);
    }
    ntstep = d.integer("ntstep", 10);
    display_freq = static_cast<int>(d.integer("display_freq", 50));
    // uniform velocity grid (generate_uniform_grid, grid/velocity_grid.f90:631-651)
    auto axis = [&](const char* n, const char* lo, const char* hi, std::vector<double>& v) {
      const int np = static_cast<int>(d.integer(n, 16));
      const double a = d.num(lo, -5.0), b = d.num(hi, 5.0);
      v.resize(np);
      for (int i = 0; i < np; ++i) v[i] = a + static_cast<double>(i) * (b - a) / static_cast<double>(np - 1);
    };
    axis("num_points_x", "xv_min", "xv_max", x);
    axis("num_points_y", "yv_min", "yv_max", y);
    axis("num_points_z", "zv_min", "zv_max", z);
    ncells = p.nx_space * p.ny_space;
    nv = static_cast<int>(x.size() * y.size() * z.size());
    return true;
  }

  // compute_beta (grid/velocity_grid.f90:486-540)
  static double beta(const std::vector<double>& a, size_t i) {
    const size_t N = a.size();
    if (i == 0) return a[1] - a[0];
    if (i == N - 1) return a[N - 1] - a[N - 2];
    return (a[i + 1] - a[i]) / 2.0 + (a[i] - a[i - 1]) / 2.0;
  }

  // One cell of initialize_dist_func (conditions/initial_conditions.f90:465-617): the
  // velocity distribution InitDF (1 Maxwellian, 2 BKW at K = 3/5, 3 a delta function at
  // {x,y,z}_delta_loc, 4 the Maxwellian integrated exactly over each node's cell) of the
  // local state, times the node volume, then scaled so that its sum is the density. A zero
  // density leaves the cell empty (:456-469).
  void fill_cell(double* out, int initdf, double n, double u, double v, double w, double T,
                 const double delta[3]) const {
    const size_t nv = x.size() * y.size() * z.size();
    if (n == 0.0) {
      for (size_t l = 0; l < nv; ++l) out[l] = 0.0;
      return;
    }
    const double pi = p.pi_mode == DVM_PI_EXACT ? kPiExact : kPiReference;
    const double mass = p.mass;
    const double opt = mass / (pi * T);
    const double maxwell_coeff = n * std::sqrt(opt * opt * opt);
    const double bkw_xk = 1.0 - 0.4 * std::exp(-0.0 / 6.0);
    const double bkw_norm = 0.5 * n * std::sqrt(opt * opt * opt) * std::pow(bkw_xk, -2.5);
    double calculated = 0.0;
    size_t l = 0;
    for (size_t k = 0; k < z.size(); ++k) {
      const double bz = beta(z, k);
      const double z1 = k > 0 ? z[k - 1] : z[k] - bz, z2 = k + 1 < z.size() ? z[k + 1] : z[k] + bz;
      for (size_t j = 0; j < y.size(); ++j) {
        const double by = beta(y, j);
        const double y1 = j > 0 ? y[j - 1] : y[j] - by, y2 = j + 1 < y.size() ? y[j + 1] : y[j] + by;
        for (size_t i = 0; i < x.size(); ++i, ++l) {
          const double bx = beta(x, i);
          const double b3 = bx * by * bz;
          double cxsq = (x[i] - u);
          cxsq = cxsq * cxsq;
          double cysq = (y[j] - v);
          cysq = cysq * cysq;
          double czsq = (z[k] - w);
          czsq = czsq * czsq;
          const double csq = cxsq + cysq + czsq;
          double df = 0.0;
          if (initdf == 1) {  // compute_maxwellian (dist_funcs/dist_func.f90:317-343)
            df = maxwell_coeff * std::exp(-csq * mass / T);
          } else if (initdf == 2) {  // compute_bkw (:374-401)
            df = bkw_norm * (5.0 * bkw_xk - 3.0 + 2.0 * (1.0 - bkw_xk) * csq * mass / (bkw_xk * T)) *
                 std::exp(-csq * mass / (bkw_xk * T));
          } else if (initdf == 3) {
            df = (std::fabs(delta[0] - x[i]) < 1.0e-13 && std::fabs(delta[1] - y[j]) < 1.0e-13 &&
                  std::fabs(delta[2] - z[k]) < 1.0e-13) ? n / b3 : 0.0;
          } else {  // compute_exact_gaussian (:345-372)
            const double x1 = i > 0 ? x[i - 1] : x[i] - bx, x2 = i + 1 < x.size() ? x[i + 1] : x[i] + bx;
            const double C2 = mass / T, sq = std::sqrt(C2);
            const double xl = sq * (x1 + 0.5 * (x[i] - x1) - u), xr = sq * (x[i] + 0.5 * (x2 - x[i]) - u);
            const double yl = sq * (y1 + 0.5 * (y[j] - y1) - v), yr = sq * (y[j] + 0.5 * (y2 - y[j]) - v);
            const double zl = sq * (z1 + 0.5 * (z[k] - z1) - w), zr = sq * (z[k] + 0.5 * (z2 - z[k]) - w);
            const double Cx = std::erf(xr) - std::erf(xl);
            const double Cy = std::erf(yl) - std::erf(yr);
            const double Cz = std::erf(zl) - std::erf(zr);
            df = 0.125 * maxwell_coeff * std::pow(pi / C2, 1.5) * Cx * Cy * Cz;
          }
          out[l] = df * b3;
          calculated = calculated + out[l];
        }
      }
    }
    const double ratio = n / calculated;
    for (size_t q = 0; q < l; ++q) out[q] = ratio * out[q];
  }

  // initialize_dist_func (conditions/initial_conditions.f90:212-650). InitC: 1 every cell in
  // the left wall's state, 2 in the right wall's, 3 the left wall's up to spatial_middle and
  // the right wall's beyond, 5 the *_init state; this build's 6 and 7 are described at the
  // top of the file. A state that comes out non-finite is refused.
  bool initial_state(const Deck& d, std::string& err) {
    f.assign(static_cast<size_t>(ncells) * nv, 0.0);
    const int initdf = static_cast<int>(d.integer("InitDF", 1));
    if (initdf < 1 || initdf > 4) { err = "InitDF " + std::to_string(initdf) + " not supported"; return false; }
    const int initc = static_cast<int>(d.integer("InitC", 5));
    const double delta[3] = {d.num("x_delta_loc", 0.0), d.num("y_delta_loc", 0.0), d.num("z_delta_loc", 0.0)};
    const long long space_mid = d.integer("spatial_middle", p.nx_space / 2);
    std::vector<double> tmp(nv);
    for (int c = 0; c < ncells; ++c) {
      double* fc = f.data() + static_cast<size_t>(c) * nv;
      const int cx = c % p.nx_space;
      if (initc == 1 || initc == 2 || initc == 3) {
        const int w = (initc == 1 || (initc == 3 && cx + 1 <= space_mid)) ? 0 : 1;
        fill_cell(fc, initdf, p.wall[w][0], p.wall[w][1], p.wall[w][2], p.wall[w][3], p.wall[w][4], delta);
      } else if (initc == 5) {
        fill_cell(fc, initdf, d.num("dens_init", 1.0), d.num("x_vel_init", 0.0), d.num("y_vel_init", 0.0),
                  d.num("z_vel_init", 0.0), d.num("tr_temp_init", 1.0), delta);
      } else if (initc == 6 && initdf == 1) {
        const double Tr = d.num("bimodal_T_ratio", 3.0), u = d.num("bimodal_drift", 1.0);
        fill_cell(fc, 1, 1.0, u, 0.0, 0.0, 1.0, delta);
        fill_cell(tmp.data(), 1, 1.0, -u, 0.0, 0.0, Tr, delta);
        for (int l = 0; l < nv; ++l) fc[l] = 0.5 * fc[l] + 0.5 * tmp[l];
      } else if (initc == 7 && initdf == 1) {
        // stationary shock, flow in -x (conditions/shock_conditions.f90:54-171)
        const double M = d.num("mach_number", 1.5), width = d.num("shock_width", 10.0);
        const double g = 5.0 / 3.0, Tu = 1.0, nu = 1.0;
        const double a_up = std::sqrt(g * Tu / (2.0 * p.mass)), u_up = -M * a_up;
        const double Tr = ((1.0 + 2.0 * g * (M * M - 1.0) / (g + 1.0)) * (2.0 + (g - 1.0) * M * M) /
                           ((g + 1.0) * M * M));
        const double nr = (g + 1.0) * M * M / (2.0 + (g - 1.0) * M * M);
        const double Md = std::sqrt((1.0 + 0.5 * (g - 1.0) * M * M) / (g * M * M - 0.5 * (g - 1.0)));
        const double Td = Tr * Tu, nd = nr * nu, ud = -std::sqrt(g * Td / (2.0 * p.mass)) * Md;
        const double xc = (cx + 0.5) * p.dx, x0 = 0.5 * p.nx_space * p.dx;
        const double sh = 0.5 * (1.0 + std::tanh((xc - x0) / width));
        fill_cell(fc, 1, nd + (nu - nd) * sh, ud + (u_up - ud) * sh, 0.0, 0.0, Td + (Tu - Td) * sh, delta);
        if (c == 0) {  // inflow states of both ends
          const double L[5] = {nd, ud, 0.0, 0.0, Td}, R[5] = {nu, u_up, 0.0, 0.0, Tu};
          for (int q = 0; q < 5; ++q) { p.wall[0][q] = L[q]; p.wall[1][q] = R[q]; }
        }
      } else if (initc == 4) {
        err = "InitC 4 (the reference's linear Rankine-Hugoniot ramp) is not supported; "
              "InitC 7 builds the shock joined by a tanh profile";
        return false;
      } else {
        err = "InitC " + std::to_string(initc) + " with InitDF " + std::to_string(initdf) +
              " not supported";
        return false;
      }
    }
    for (double v : f)
      if (!std::isfinite(v)) {
        err = "the initial state is not finite (InitC " + std::to_string(initc) +
              ": check the density and temperature it takes)";
        return false;
      }
    return true;
  }

  int initialize_solver() {
    dvm_vgrid vg{static_cast<int32_t>(x.size()), static_cast<int32_t>(y.size()),
                 static_cast<int32_t>(z.size()), x.data(), y.data(), z.data()};
    int st = dvm_create(&p, &vg, &ctx);
    if (st) return st;
    return dvm_upload_f(ctx, f.data());
  }

  // print_property_update (input_output/screen_output.f90:146-207), cell 0
  void print_update(long long ntime) {
    std::vector<double> props(static_cast<size_t>(ncells) * DVM_NPROP);
    int64_t colls = 0;
    dvm_get_properties(ctx, props.data());
    dvm_last_collision_count(ctx, &colls);
    std::printf("%8lld %12.5e %18.10e %18.10e %18.10e %12lld\n", ntime, ntime * p.dt,
                props[DVM_P_DENS], props[DVM_P_U], props[DVM_P_TEMP],
                static_cast<long long>(colls));
  }

  // Output (input_output/visualization.f90): the deck's [vis] settings, written through
  // dvm_vis_* from f downloaded at each output time.
  dvm_vis vis{};
  bool vis_props = false, vis_df = false;
  long long props_freq = 1, df_freq = 1;

  bool read_vis(const Deck& d, std::string& err) {
    std::memset(&vis, 0, sizeof(vis));
    static const char* keys[DVM_VIS_NPROP] = {
        "write_dens", "write_x_vel", "write_y_vel", "write_z_vel", "write_speed", "write_mach",
        "write_tr_temp", "write_rot_temp", "write_vib_temp", "write_tot_temp", "write_temp_x",
        "write_temp_y", "write_temp_z", "write_tr_energy", "write_rot_energy",
        "write_vib_energy", "write_tot_energy", "write_entropy", "write_heat_flux_x",
        "write_heat_flux_y", "write_heat_flux_z", "write_rot_dof", "write_vib_dof",
        "write_rot_temp_relax", "write_vib_temp_relax", "write_kin_temp_relax",
        "write_pressure"};
    vis_props = d.integer("enable_properties_vis", 0) != 0;
    vis_df = d.integer("enable_vel_df_vis", 0) != 0 || d.integer("enable_rot_df_vis", 0) != 0 ||
             d.integer("enable_vib_df_vis", 0) != 0;
    auto name = [&](const char* key, const char* def, char* out) {
      const std::string v = d.str(key, def);
      if (v.size() >= 128) return false;
      std::memcpy(out, v.c_str(), v.size() + 1);
      return true;
    };
    if (!name("properties_vis_filename", "properties", vis.properties_filename) ||
        !name("df_vis_filename", "dist_func", vis.df_filename)) {
      err = "output file name longer than 127 characters";
      return false;
    }
    vis.enable_properties = vis_props ? 1 : 0;
    for (int i = 0; i < DVM_VIS_NPROP; ++i)
      vis.properties_to_output[i] = d.integer(keys[i], 0) != 0 ? 1 : 0;
    const std::vector<long long> sd = d.integers("stress_directions");
    vis.write_stress = static_cast<int32_t>(d.integer("write_stress", 0));
    if (vis.write_stress < 0 || vis.write_stress > 6 ||
        static_cast<long long>(sd.size()) < vis.write_stress) {
      err = "write_stress needs that many stress_directions (at most 6)";
      return false;
    }
    for (int i = 0; i < vis.write_stress; ++i) vis.stress_directions[i] = static_cast<int32_t>(sd[i]);
    const std::vector<long long> mn = d.integers("moment_numbers");
    vis.write_moment = static_cast<int32_t>(d.integer("write_moment", 0));
    if (vis.write_moment < 0 || vis.write_moment > 6 ||
        static_cast<long long>(mn.size()) < vis.write_moment) {
      err = "write_moment needs that many moment_numbers (at most 6)";
      return false;
    }
    for (int i = 0; i < vis.write_moment; ++i) vis.moment_numbers[i] = static_cast<int32_t>(mn[i]);
    vis.nx_space = p.nx_space;
    vis.ny_space = p.ny_space;
    vis.dx = p.dx;
    vis.dy = p.dy;
    vis.end_time = static_cast<int32_t>(ntstep);
    props_freq = std::max(1LL, d.integer("properties_vis_dump_freq", 1));
    df_freq = std::max(1LL, d.integer("df_vis_dump_freq", 1));
    vis.properties_dump_freq = static_cast<int32_t>(props_freq);
    vis.enable_vel_df = d.integer("enable_vel_df_vis", 0) != 0;
    vis.enable_rot_df = d.integer("enable_rot_df_vis", 0) != 0;
    vis.enable_vib_df = d.integer("enable_vib_df_vis", 0) != 0;
    vis.df_dimension = static_cast<int32_t>(d.integer("df_output_dimension", DVM_VIS_DF_1D));
    const std::vector<long long> xl = d.integers("x_output_locations"),
                                 yl = d.integers("y_output_locations");
    vis.num_locations = static_cast<int32_t>(d.integer("num_output_locations", 0));
    if (vis_df && (vis.num_locations < 1 || vis.num_locations > 16 ||
                   static_cast<long long>(xl.size()) < vis.num_locations ||
                   static_cast<long long>(yl.size()) < vis.num_locations)) {
      err = "distribution-function output needs 1 to 16 x/y_output_locations";
      return false;
    }
    for (int i = 0; i < vis.num_locations && i < 16; ++i) {
      vis.x_locations[i] = static_cast<int32_t>(xl[i]);
      vis.y_locations[i] = static_cast<int32_t>(yl[i]);
    }
    vis.rot_levels = static_cast<int32_t>(d.integer("num_rot_levels", 0));
    vis.vib_levels = static_cast<int32_t>(d.integer("num_vib_levels", 0));
    vis.pi_mode = p.pi_mode;
    vis.mass = p.mass;
    vis.omega = p.omega;
    vis.right_wall_dens = p.wall[DVM_WALL_RIGHT][DVM_WP_DENS];
    vis.right_wall_temp_rot = d.num("rot_temp_RW", 0.0);
    vis.right_wall_temp_vib = d.num("vib_temp_RW", 0.0);
    return true;
  }

  // write_vis_data (visualization.f90:870-918): at ntime = 0, every dump_freq steps and at
  // the last step, time = ntime * deltat
  int write_vis(long long ntime, bool headers) {
    if (!vis_props && !vis_df) return DVM_OK;
    int st = DVM_OK;
    if (headers && (st = dvm_vis_write_headers(&vis))) return st;
    const bool last = ntime % std::max(1LL, ntstep) == 0;
    const bool want_props = vis_props && (last || ntime % props_freq == 0);
    const bool want_df = vis_df && (last || ntime % df_freq == 0);
    if (!want_props && !want_df) return DVM_OK;
    std::vector<double> fh(static_cast<size_t>(ncells) * nv);
    if ((st = dvm_download_f(ctx, fh.data()))) return st;
    dvm_vgrid vg{static_cast<int32_t>(x.size()), static_cast<int32_t>(y.size()),
                 static_cast<int32_t>(z.size()), x.data(), y.data(), z.data()};
    const double time = static_cast<double>(ntime) * p.dt;
    if (want_df && (st = dvm_vis_write_df(&vis, time, fh.data(), &vg))) return st;
    if (want_props && (st = dvm_vis_write_properties(&vis, time, nullptr, fh.data(), &vg))) return st;
    return DVM_OK;
  }

  // solve (solver/dvm_solver.f90:231-369)
  int solve(long long nsteps, long long first = 0) {
    std::printf("%8s %12s %18s %18s %18s %12s\n", "ntime", "time", "dens", "x_vel", "temp", "colls");
    for (long long ntime = first + 1; ntime <= first + nsteps; ++ntime) {
      int st = dvm_compute_collision_integral(ctx, static_cast<uint64_t>(ntime - 1), nullptr);
      if (!st) st = dvm_compute_convection(ctx);
      if (!st) st = dvm_calculate_physical_properties(ctx);
      if (st) return st;
      if (ntime % display_freq == 0 || ntime == first + nsteps) print_update(ntime);
      if ((st = write_vis(ntime, false))) return st;
    }
    uint32_t word = 0;
    dvm_get_error_word(ctx, &word);
    return word ? DVM_ERR_NUMERIC : DVM_OK;
  }

  void destroy_solver() {
    if (ctx) dvm_destroy(ctx);
    ctx = nullptr;
  }
};

bool read_file(const char* path, std::vector<char>& v) {
  FILE* fp = std::fopen(path, "rb");
  if (!fp) return false;
  std::fseek(fp, 0, SEEK_END);
  const long n = std::ftell(fp);
  std::fseek(fp, 0, SEEK_SET);
  v.resize(n > 0 ? static_cast<size_t>(n) : 0);
  const size_t got = v.empty() ? 0 : std::fread(v.data(), 1, v.size(), fp);
  std::fclose(fp);
  return got == v.size();
}

bool write_doubles(const char* path, const std::vector<double>& v) {
  FILE* fp = std::fopen(path, "wb");
  if (!fp) return false;
  const size_t n = std::fwrite(v.data(), sizeof(double), v.size(), fp);
  std::fclose(fp);
  return n == v.size();
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s <input deck> [--check] [--steps N] [--dump-f FILE] "
                         "[--dump-props FILE] [--restart-in FILE] [--restart-out FILE]\n",
                 argv[0]);
    return 1;
  }
  bool check = false;
  long long steps = -1;
  const char* dump_f = nullptr;
  const char* dump_props = nullptr;
  const char* restart_in = nullptr;
  const char* restart_out = nullptr;
  for (int a = 2; a < argc; ++a) {
    if (!std::strcmp(argv[a], "--check")) check = true;
    else if (!std::strcmp(argv[a], "--steps") && a + 1 < argc) steps = std::atoll(argv[++a]);
    else if (!std::strcmp(argv[a], "--dump-f") && a + 1 < argc) dump_f = argv[++a];
    else if (!std::strcmp(argv[a], "--dump-props") && a + 1 < argc) dump_props = argv[++a];
    else if (!std::strcmp(argv[a], "--restart-in") && a + 1 < argc) restart_in = argv[++a];
    else if (!std::strcmp(argv[a], "--restart-out") && a + 1 < argc) restart_out = argv[++a];
  }
  Deck deck;
  if (!deck.load(argv[1])) { std::fprintf(stderr, "Error: cannot read %s\n", argv[1]); return 1; }
  Host h;
  std::string err;
  if (!h.read_input(deck, err) || !h.initial_state(deck, err) || !h.read_vis(deck, err)) {
    std::fprintf(stderr, "Error: %s\n", err.c_str());
    return 1;
  }
  if (steps < 0) steps = h.ntstep;
  if (check) {
    double mass = 0.0;
    for (double v : h.f) mass += v;
    std::printf("geometry %d cells %d nv %d coll %d conv %d sigma %.17g omega %.17g alpha %.17g "
                "dt %.17g Kn %.17g samples_mode %d samples %lld steps %lld mass %.17g\n",
                h.p.geometry, h.ncells, h.nv, h.p.coll_method, h.p.conv_method, h.p.sigma,
                h.p.omega, h.p.alpha, h.p.dt, h.p.Kn, h.p.samples_mode,
                static_cast<long long>(h.p.samples_per_step), steps, mass);
    if (mass == 0.0)
      std::fprintf(stderr, "warning: the initial state is empty (the density InitC takes is 0)\n");
    if (dump_f && !write_doubles(dump_f, h.f)) {  // the initial state, no device needed
      std::fprintf(stderr, "Error: cannot write %s\n", dump_f);
      return 1;
    }
    return 0;
  }
  int st = h.initialize_solver();
  long long first = 0;
  if (!st && restart_in) {  // continue a saved run (restart.f90: ntime and phi)
    std::vector<char> buf;
    uint64_t nt = 0;
    if (!read_file(restart_in, buf)) st = DVM_ERR_PARAM;
    if (!st) st = dvm_checkpoint_load(h.ctx, buf.data(), buf.size(), &nt);
    first = static_cast<long long>(nt);
  }
  if (!st) st = h.write_vis(first, true);
  if (!st) st = h.solve(steps, first);
  if (!st && restart_out) {
    uint64_t n = 0;
    st = dvm_checkpoint_size(h.ctx, &n);
    std::vector<char> buf(n);
    if (!st) st = dvm_checkpoint_save(h.ctx, static_cast<uint64_t>(first + steps), buf.data(), n);
    FILE* fp = st ? nullptr : std::fopen(restart_out, "wb");
    if (!st && (!fp || std::fwrite(buf.data(), 1, n, fp) != n)) st = DVM_ERR_PARAM;
    if (fp) std::fclose(fp);
  }
  if (!st && dump_f) {
    std::vector<double> out(h.f.size());
    st = dvm_download_f(h.ctx, out.data());
    if (!st && !write_doubles(dump_f, out)) st = DVM_ERR_PARAM;
  }
  if (!st && dump_props) {
    std::vector<double> out(static_cast<size_t>(h.ncells) * DVM_NPROP);
    st = dvm_get_properties(h.ctx, out.data());
    if (!st && !write_doubles(dump_props, out)) st = DVM_ERR_PARAM;
  }
  h.destroy_solver();
  if (st) {
    std::fprintf(stderr, "Error: %s\n", dvm_strerror(st));  // the reference prints and stops
    return 2;
  }
  return 0;
}
