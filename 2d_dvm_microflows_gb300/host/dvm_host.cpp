// dvm_host.cpp -- C++ host of the GPU time step: the reference driver's program flow
// (main.f90:25-38: initialize_solver, solve, destroy_solver in solver/dvm_solver.f90)
// running through the C ABI of include/dvm_gpu.h.
//
//   dvm_host <input deck> [--check] [--steps N] [--dump-f FILE] [--dump-props FILE]
//
// The deck is the reference's `key = value` format (input_output/read_input_2D.f90:75-777;
// e.g. trunk/bin/velocity_refined.inp): [sections] and `#` comments are skipped, values may
// be quoted and may use Fortran exponents (1.0d0). Keys read: Kn, species_codes,
// csection_method, csection_coeff, delta_x, delta_y, nx_space, ny_space, deltat, ntstep,
// num_points_{x,y,z}, {x,y,z}v_{min,max}, InitC, InitDF, dens_init, {x,y,z}_vel_init,
// tr_temp_init, {dens,x_vel,y_vel,z_vel,tr_temp}_{LW,RW,BW,TW}, {L,R,B,T}WallBC,
// acc_coeff, iColl, cdf_tolerance, NRepl, ColnRMS, iConv, display_freq. Keys this build
// adds: geometry, samples_per_step, seed, pi_mode, and for the initial states of the
// benchmark configurations InitC = 6 (two drifting Maxwellians: bimodal_T_ratio,
// bimodal_drift) and InitC = 7 (Rankine-Hugoniot shock joined by a tanh profile:
// mach_number, shock_width).
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
    p.nx_space = static_cast<int>(d.integer("nx_space", 1));
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

  // Discrete Maxwellian times the node volume, renormalised to n
  // (conditions/initial_conditions.f90:480-617).
  void maxwellian(double* out, double n, double u, double v, double w, double T) const {
    const double pi = p.pi_mode == DVM_PI_EXACT ? kPiExact : kPiReference;
    auto beta = [](const std::vector<double>& a, size_t i) {
      const size_t N = a.size();
      if (i == 0) return a[1] - a[0];
      if (i == N - 1) return a[N - 1] - a[N - 2];
      return (a[i + 1] - a[i]) / 2.0 + (a[i] - a[i - 1]) / 2.0;
    };
    const double opt = p.mass / (pi * T);
    const double coeff = n * std::sqrt(opt * opt * opt);
    double sum = 0.0;
    size_t l = 0;
    for (size_t k = 0; k < z.size(); ++k)
      for (size_t j = 0; j < y.size(); ++j)
        for (size_t i = 0; i < x.size(); ++i, ++l) {
          const double c2 = (x[i] - u) * (x[i] - u) + (y[j] - v) * (y[j] - v) + (z[k] - w) * (z[k] - w);
          out[l] = coeff * std::exp(-c2 * p.mass / T) * beta(x, i) * beta(y, j) * beta(z, k);
          sum += out[l];
        }
    if (sum > 0.0)
      for (size_t q = 0; q < l; ++q) out[q] = (n / sum) * out[q];
  }

  // initialize_dist_func (conditions/initial_conditions.f90:212-650), Maxwellian states.
  bool initial_state(const Deck& d, std::string& err) {
    f.assign(static_cast<size_t>(ncells) * nv, 0.0);
    if (d.integer("InitDF", 1) != 1) { err = "only InitDF = 1 (Maxwellian) is supported"; return false; }
    const int initc = static_cast<int>(d.integer("InitC", 5));
    std::vector<double> tmp(nv);
    for (int c = 0; c < ncells; ++c) {
      double* fc = f.data() + static_cast<size_t>(c) * nv;
      const int cx = c % p.nx_space;
      if (initc == 1 || initc == 2 || initc == 3) {
        const int w = (initc == 1 || (initc == 3 && cx < p.nx_space / 2)) ? 0 : 1;
        maxwellian(fc, p.wall[w][0], p.wall[w][1], p.wall[w][2], p.wall[w][3], p.wall[w][4]);
      } else if (initc == 5) {
        maxwellian(fc, d.num("dens_init", 1.0), d.num("x_vel_init", 0.0), d.num("y_vel_init", 0.0),
                   d.num("z_vel_init", 0.0), d.num("tr_temp_init", 1.0));
      } else if (initc == 6) {
        const double Tr = d.num("bimodal_T_ratio", 3.0), u = d.num("bimodal_drift", 1.0);
        maxwellian(fc, 1.0, u, 0.0, 0.0, 1.0);
        maxwellian(tmp.data(), 1.0, -u, 0.0, 0.0, Tr);
        for (int l = 0; l < nv; ++l) fc[l] = 0.5 * fc[l] + 0.5 * tmp[l];
      } else if (initc == 7) {
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
        const double s = 0.5 * (1.0 + std::tanh((xc - x0) / width));
        maxwellian(fc, nd + (nu - nd) * s, ud + (u_up - ud) * s, 0.0, 0.0, Td + (Tu - Td) * s);
        if (c == 0) {  // inflow states of both ends
          const double L[5] = {nd, ud, 0.0, 0.0, Td}, R[5] = {nu, u_up, 0.0, 0.0, Tu};
          for (int q = 0; q < 5; ++q) { p.wall[0][q] = L[q]; p.wall[1][q] = R[q]; }
        }
      } else {
        err = "InitC " + std::to_string(initc) + " not supported";
        return false;
      }
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

  // solve (solver/dvm_solver.f90:231-369)
  // Tecplot output of the moments in the layout of write_properties
  // (input_output/visualization.f90:620-660, 1591-1660).
  const char* props_dat = nullptr;
  long long props_every = 1;

  void write_props_header() const {
    FILE* fp = std::fopen(props_dat, "w");
    if (!fp) return;
    std::fprintf(fp, "title = \"Macroscopic Properties\"\n");
    std::fprintf(fp, "variables = \"Time\", \"x-Location\", \"y-Location\", \"Density\", "
                     "\"X-Velocity\", \"Y-Velocity\", \"Z-Velocity\", \"Temperature\", "
                     "\"Avg Speed\", \"Pressure\", \"Heat Flux X\", \"Heat Flux Y\", "
                     "\"Heat Flux Z\", \"Tau xx\", \"Tau yy\", \"Tau zz\", \"Tau xy\", "
                     "\"Tau xz\", \"Tau yz\"\n");
    std::fclose(fp);
  }

  int write_props(long long ntime) const {
    std::vector<double> pr(static_cast<size_t>(ncells) * DVM_NPROP);
    int st = dvm_get_properties(ctx, pr.data());
    if (st) return st;
    FILE* fp = std::fopen(props_dat, "a");
    if (!fp) return DVM_ERR_PARAM;
    static const int cols[] = {DVM_P_DENS, DVM_P_U, DVM_P_V, DVM_P_W, DVM_P_TEMP, DVM_P_AVG_SPEED,
                               DVM_P_PRESSURE, DVM_P_QX, DVM_P_QY, DVM_P_QZ, DVM_P_TXX, DVM_P_TYY,
                               DVM_P_TZZ, DVM_P_TXY, DVM_P_TXZ, DVM_P_TYZ};
    std::fprintf(fp, "zone i=%5d\n", ncells);
    const double time = static_cast<double>(ntime) * p.dt;
    for (int cx = 0; cx < p.nx_space; ++cx)
      for (int cy = 0; cy < p.ny_space; ++cy) {
        const double* q = pr.data() + static_cast<size_t>(cx + p.nx_space * cy) * DVM_NPROP;
        std::fprintf(fp, "%24.15e%24.15e%24.15e", time, (cx + 0.5) * p.dx, (cy + 0.5) * p.dy);
        for (int c : cols) std::fprintf(fp, "%24.15e", q[c]);
        std::fprintf(fp, "\n");
      }
    std::fclose(fp);
    return DVM_OK;
  }

  int solve(long long nsteps, long long first = 0) {
    std::printf("%8s %12s %18s %18s %18s %12s\n", "ntime", "time", "dens", "x_vel", "temp", "colls");
    for (long long ntime = first + 1; ntime <= first + nsteps; ++ntime) {
      int st = dvm_compute_collision_integral(ctx, static_cast<uint64_t>(ntime - 1), nullptr);
      if (!st) st = dvm_compute_convection(ctx);
      if (!st) st = dvm_calculate_physical_properties(ctx);
      if (st) return st;
      if (ntime % display_freq == 0 || ntime == first + nsteps) print_update(ntime);
      if (props_dat && (ntime % props_every == 0 || ntime == first + nsteps)) {
        st = write_props(ntime);
        if (st) return st;
      }
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
                         "[--dump-props FILE] [--props-dat FILE] [--props-every N] "
                         "[--restart-in FILE] [--restart-out FILE]\n", argv[0]);
    return 1;
  }
  bool check = false;
  long long steps = -1;
  const char* dump_f = nullptr;
  const char* dump_props = nullptr;
  const char* props_dat = nullptr;
  const char* restart_in = nullptr;
  const char* restart_out = nullptr;
  long long props_every = 1;
  for (int a = 2; a < argc; ++a) {
    if (!std::strcmp(argv[a], "--check")) check = true;
    else if (!std::strcmp(argv[a], "--steps") && a + 1 < argc) steps = std::atoll(argv[++a]);
    else if (!std::strcmp(argv[a], "--dump-f") && a + 1 < argc) dump_f = argv[++a];
    else if (!std::strcmp(argv[a], "--dump-props") && a + 1 < argc) dump_props = argv[++a];
    else if (!std::strcmp(argv[a], "--props-dat") && a + 1 < argc) props_dat = argv[++a];
    else if (!std::strcmp(argv[a], "--props-every") && a + 1 < argc) props_every = std::atoll(argv[++a]);
    else if (!std::strcmp(argv[a], "--restart-in") && a + 1 < argc) restart_in = argv[++a];
    else if (!std::strcmp(argv[a], "--restart-out") && a + 1 < argc) restart_out = argv[++a];
  }
  Deck deck;
  if (!deck.load(argv[1])) { std::fprintf(stderr, "Error: cannot read %s\n", argv[1]); return 1; }
  Host h;
  std::string err;
  if (!h.read_input(deck, err) || !h.initial_state(deck, err)) {
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
  h.props_dat = props_dat;
  h.props_every = props_every > 0 ? props_every : 1;
  if (!st && props_dat) {
    h.write_props_header();
    st = h.write_props(first);
  }
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
