// Init.txt readers of the C ABI: the reference's 17 positional values
// (kernel.cu:1705-1723) and the extension lines after them.
#include "ds_inittxt.cuh"

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <utility>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// Init.txt: the reference's 17 positional values (kernel.cu:1705-1723), then
// extension lines "name = value" ("//" starts a comment, lines without "=" are
// skipped).  The reference stops reading after line 18, so an extended file
// still runs it.
// ---------------------------------------------------------------------------
std::string trim(const std::string &t) {
  size_t a = 0, b = t.size();
  while (a < b && isspace((unsigned char)t[a])) a++;
  while (b > a && isspace((unsigned char)t[b - 1])) b--;
  return t.substr(a, b - a);
}

std::string lower(std::string t) {
  for (auto &ch : t) ch = (char)tolower((unsigned char)ch);
  return t;
}

bool parse_double(const std::string &v, double *out) {
  const std::string t = trim(v);
  if (t.empty()) return false;
  char *end = nullptr;
  const double d = strtod(t.c_str(), &end);
  if (end != t.c_str() + t.size()) return false;
  *out = d;
  return true;
}

bool parse_int(const std::string &v, int *out) {
  const std::string t = trim(v);
  if (t.empty()) return false;
  char *end = nullptr;
  const long x = strtol(t.c_str(), &end, 10);
  if (end != t.c_str() + t.size() || x < -2147483647L - 1 || x > 2147483647L) return false;
  *out = (int)x;
  return true;
}

// The extension lines of a file: (key, value) in file order, after line 18.
bool extension_lines(const char *path, std::vector<std::pair<std::string, std::string>> &kv) {
  FILE *f = fopen(path, "r");
  if (!f) return false;
  std::string line;
  int lineno = 0, ch;
  auto flush = [&]() {
    if (++lineno > 18) {
      std::string body = line.substr(0, line.find("//"));
      body = trim(body);
      const size_t eq = body.find('=');
      if (!body.empty() && eq != std::string::npos)
        kv.emplace_back(trim(body.substr(0, eq)), trim(body.substr(eq + 1)));
    }
    line.clear();
  };
  while ((ch = fgetc(f)) != EOF) {
    if (ch == '\n' || ch == '\r') {
      if (ch == '\r') {  // \r\n is one line end
        const int nx = fgetc(f);
        if (nx != '\n' && nx != EOF) ungetc(nx, f);
      }
      flush();
    } else {
      line.push_back((char)ch);
    }
  }
  if (!line.empty()) flush();
  fclose(f);
  return true;
}

struct ModeName {
  const char *name;
  int bit;
};
const ModeName kModeNames[] = {
    {"periodic_y", DS_MODE_PERIODIC_Y}, {"periodic_z", DS_MODE_PERIODIC_Z},
    {"h_per_particle", DS_MODE_H_PER_PARTICLE}, {"tstop_const", DS_MODE_TSTOP_CONST},
    {"gas_accel_particle", DS_MODE_GAS_ACCEL_PARTICLE}, {"ref_index_coupling", DS_MODE_REF_INDEX_COUPLING},
    {"ref_eps_guard", DS_MODE_REF_EPS_GUARD}, {"ref_solve2", DS_MODE_REF_SOLVE2}, {"cfl", DS_MODE_CFL},
    {"dust_rho", DS_MODE_DUST_RHO}, {"grid_proper", DS_MODE_GRID_PROPER}, {"idic_proper", DS_MODE_IDIC_PROPER}};

ds_status apply_param_extension(ds_params *p, const std::string &key, const std::string &val) {
  if (key == "ic" || key.rfind("ic.", 0) == 0) return DS_OK;  // initial conditions: ds_ic_read_init_txt
  if (key.rfind("mode.", 0) == 0) {
    const std::string name = key.substr(5), v = lower(trim(val));
    const bool on = v == "1" || v == "true" || v == "yes" || v == "on";
    for (const ModeName &m : kModeNames)
      if (name == m.name) {
        p->mode = on ? (p->mode | m.bit) : (p->mode & ~m.bit);
        return DS_OK;
      }
    return DS_ERR_ARG;
  }
  double *lists[] = {p->mass_ratio, p->R_dust, p->t_stop_const, p->eps_empty};
  const char *list_names[] = {"mass_ratio", "R_dust", "t_stop_const", "eps_empty"};
  for (int l = 0; l < 4; l++)
    if (key == list_names[l]) {  // values separated by spaces or commas; missing entries 0
      std::string t = val;
      for (auto &ch : t) if (ch == ',') ch = ' ';
      double vals[DS_MAX_DUST] = {};
      size_t pos = 0;
      int k = 0;
      while (true) {
        while (pos < t.size() && isspace((unsigned char)t[pos])) pos++;
        if (pos >= t.size()) break;
        size_t e = pos;
        while (e < t.size() && !isspace((unsigned char)t[e])) e++;
        double d;
        if (!parse_double(t.substr(pos, e - pos), &d)) return DS_ERR_ARG;
        if (k < DS_MAX_DUST) vals[k] = d;
        k++;
        pos = e;
      }
      for (int q = 0; q < DS_MAX_DUST; q++) lists[l][q] = vals[q];
      return DS_OK;
    }
  int *ints[] = {&p->n_dust, &p->stencil, &p->list_depth, &p->force_list, &p->persistent, &p->idic_lanes};
  const char *int_names[] = {"n_dust", "stencil", "list_depth", "force_list", "persistent", "idic_lanes"};
  for (int q = 0; q < 6; q++)
    if (key == int_names[q]) return parse_int(val, ints[q]) ? DS_OK : DS_ERR_ARG;
  if (key == "precision") {
    const std::string v = lower(trim(val));
    p->precision = (v == "fp32" || v == "1") ? DS_PRECISION_FP32 : DS_PRECISION_FP64;
    return DS_OK;
  }
  struct DName {
    const char *name;
    double *d;
  };
  const DName dn[] = {{"X_min", &p->X_min}, {"X_max", &p->X_max}, {"Y_min", &p->Y_min}, {"Y_max", &p->Y_max},
                      {"Z_min", &p->Z_min}, {"Z_max", &p->Z_max}, {"Particle_on_length", &p->Particle_on_length},
                      {"h", &p->h}, {"Coeff_h_dust_cell", &p->Coeff_h_dust_cell}, {"tau", &p->tau},
                      {"T_end", &p->T_end}, {"T_out", &p->T_out}, {"alpha", &p->alpha}, {"beta", &p->beta},
                      {"eps", &p->eps}, {"Gam_g", &p->Gam_g}, {"Speed_of_sound_gas", &p->Speed_of_sound_gas},
                      {"t_empty", &p->t_empty}, {"cell_w", &p->cell_w}, {"idic_w", &p->idic_w}, {"cfl", &p->cfl},
                      {"list_skin", &p->list_skin}};
  for (const DName &d : dn)
    if (key == d.name) return parse_double(val, d.d) ? DS_OK : DS_ERR_ARG;
  if (key == "Type_of_state" || key == "Maximum_particle") {  // numbers, truncated to int
    double d;
    if (!parse_double(val, &d) || !(std::fabs(d) < 2147483648.0)) return DS_ERR_ARG;
    (key == "Type_of_state" ? p->Type_of_state : p->Maximum_particle) = (int)d;
    return DS_OK;
  }
  return DS_ERR_ARG;  // unknown name
}

}  // namespace

ds_status ds_read_init_txt_file(const char *path, ds_params *p) {
  FILE *f = fopen(path, "r");
  if (!f) return DS_ERR_ARG;
  char s[256];
  if (!fgets(s, sizeof s, f)) { fclose(f); return DS_ERR_ARG; }
  double *dv[] = {&p->X_min, &p->X_max, &p->Y_min, &p->Y_max, &p->Z_min, &p->Z_max};
  int ok = 1;
  for (double *d : dv) ok &= fgets(s, sizeof s, f) && sscanf(s, "%lf", d) == 1;
  ok &= fgets(s, sizeof s, f) && sscanf(s, "%d", &p->Type_of_state) == 1;
  ok &= fgets(s, sizeof s, f) && sscanf(s, "%d", &p->Maximum_particle) == 1;
  double *dv2[] = {&p->Particle_on_length, &p->h, &p->Coeff_h_dust_cell, &p->tau, &p->T_end,
                   &p->T_out, &p->alpha, &p->beta, &p->eps};
  for (double *d : dv2) ok &= fgets(s, sizeof s, f) && sscanf(s, "%lf", d) == 1;
  fclose(f);
  if (!ok) return DS_ERR_ARG;
  std::vector<std::pair<std::string, std::string>> kv;
  if (!extension_lines(path, kv)) return DS_ERR_ARG;
  for (const auto &e : kv)
    if (apply_param_extension(p, e.first, e.second) != DS_OK) return DS_ERR_ARG;
  return DS_OK;
}

// "ic = sod_x_dust | sod_x_mas | dusty_sod" and "ic.<field> = value" lines.
ds_status ds_read_ic_txt_file(const char *path, ds_ic *ic) {
  std::vector<std::pair<std::string, std::string>> kv;
  if (!extension_lines(path, kv)) return DS_ERR_ARG;
  int kind = DS_IC_SOD_X_DUST;  // the generator the reference's main calls
  for (const auto &e : kv)
    if (e.first == "ic") {
      const std::string v = lower(e.second);
      if (v == "sod_x_dust") kind = DS_IC_SOD_X_DUST;
      else if (v == "sod_x_mas") kind = DS_IC_SOD_X_MAS;
      else if (v == "dusty_sod") kind = DS_IC_DUSTY_SOD;
      else return DS_ERR_ARG;
    }
  ds_ic_init(ic, kind);
  struct DName {
    const char *name;
    double *d;
  };
  const DName dn[] = {{"dx_left", &ic->dx_left}, {"Ly", &ic->Ly}, {"Lz", &ic->Lz}, {"eps", &ic->eps},
                      {"t_s", &ic->t_s}, {"rho_L", &ic->rho_L}, {"p_L", &ic->p_L}, {"rho_R", &ic->rho_R},
                      {"p_R", &ic->p_R}, {"gamma", &ic->gamma}, {"h_factor", &ic->h_factor}, {"x0", &ic->x0},
                      {"x1", &ic->x1}, {"wall", &ic->wall}, {"lattice_offset", &ic->lattice_offset},
                      {"t_end", &ic->t_end}, {"cfl", &ic->cfl}, {"alpha", &ic->alpha}, {"beta", &ic->beta},
                      {"av_eps", &ic->av_eps}, {"idic_cells", &ic->idic_cells}, {"fixed_tau", &ic->fixed_tau}};
  for (const auto &e : kv) {
    if (e.first.rfind("ic.", 0) != 0) continue;
    const std::string name = e.first.substr(3);
    bool found = false;
    for (const DName &d : dn)
      if (name == d.name) {
        if (!parse_double(e.second, d.d)) return DS_ERR_ARG;
        found = true;
      }
    if (!found) return DS_ERR_ARG;
  }
  return DS_OK;
}
