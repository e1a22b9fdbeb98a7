// sph_problem.cpp -- host-side problem set-up (reference-format reader and synthetic
// generators).  Restates the reference's set-up routines of
// example_problems/soil_failure_bui_et_al_2008/3_SPH_material_2018.f90 (problem_input_data
// :37-340, setup_particles :344, Read_2DMesh :365-751, set_up_dummy_nodes :755-897,
// Setup_Global_Arrays :902-1045, Get_BCs_on_node :1049-1131, Initial_conditions
// :1433-1569) with the same FP32 roundings (`real` locals become float).
#include <cerrno>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../../include/sph_host.h"

namespace {

struct ParseError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// Fortran list-directed input over one file: a READ statement consumes values from as many
// records as it needs and then skips the rest of its last record.
class ListReader {
 public:
  ListReader(const std::string& text, std::string name) : name_(std::move(name)) {
    std::string line;
    std::istringstream is(text);
    while (std::getline(is, line)) lines_.push_back(line);
  }
  // values of one READ statement
  std::vector<std::string> read(size_t n) {
    std::vector<std::string> out;
    while (out.size() < n) {
      if (rec_ >= lines_.size())
        throw ParseError(name_ + ": end of file while reading record " + std::to_string(rec_ + 1));
      const std::string& l = lines_[rec_++];
      size_t i = 0;
      while (i < l.size() && out.size() < n) {
        while (i < l.size() && (l[i] == ' ' || l[i] == '\t' || l[i] == ',' || l[i] == '\r')) i++;
        if (i >= l.size()) break;
        size_t j = i;
        if (l[i] == '\'' || l[i] == '"') {
          char q = l[i];
          j = i + 1;
          while (j < l.size() && l[j] != q) j++;
          out.push_back(l.substr(i + 1, j - i - 1));
          i = j + 1;
          continue;
        }
        while (j < l.size() && l[j] != ' ' && l[j] != '\t' && l[j] != ',' && l[j] != '\r') j++;
        out.push_back(l.substr(i, j - i));
        i = j;
      }
    }
    return out;
  }
  // number of value tokens on the next non-blank record (does not consume it)
  size_t peek_count() const {
    size_t r = rec_;
    while (r < lines_.size()) {
      std::string t;
      size_t n = 0;
      std::string l = lines_[r];
      for (char& ch : l)
        if (ch == ',' || ch == '\t' || ch == '\r') ch = ' ';
      std::istringstream is2(l);
      while (is2 >> t) {
        if (t[0] == '!') break;
        n++;
      }
      if (n) return n;
      r++;
    }
    return 0;
  }
  void text() { read(1); }
  double dbl() { return to_d(read(1)[0]); }
  int integer() { return to_i(read(1)[0]); }
  bool logical() { return to_l(read(1)[0]); }
  double to_d(std::string s) const {
    for (char& ch : s)
      if (ch == 'd' || ch == 'D') ch = 'e';
    char* e = nullptr;
    errno = 0;
    double v = std::strtod(s.c_str(), &e);
    if (e == s.c_str() || *e) throw ParseError(name_ + ": bad real '" + s + "'");
    return v;
  }
  float to_f(std::string s) const {
    for (char& ch : s)
      if (ch == 'd' || ch == 'D') ch = 'e';
    char* e = nullptr;
    float v = std::strtof(s.c_str(), &e);
    if (e == s.c_str() || *e) throw ParseError(name_ + ": bad real '" + s + "'");
    return v;
  }
  int to_i(const std::string& s) const {
    char* e = nullptr;
    long v = std::strtol(s.c_str(), &e, 10);
    if (e == s.c_str() || *e) throw ParseError(name_ + ": bad integer '" + s + "'");
    return (int)v;
  }
  bool to_l(const std::string& s) const {
    size_t i = (s.size() && s[0] == '.') ? 1 : 0;
    if (i < s.size() && (s[i] == 'T' || s[i] == 't')) return true;
    if (i < s.size() && (s[i] == 'F' || s[i] == 'f')) return false;
    throw ParseError(name_ + ": bad logical '" + s + "'");
  }

 private:
  std::vector<std::string> lines_;
  size_t rec_ = 0;
  std::string name_;
};

}  // namespace

struct sph_problem {
  std::string name;
  sps_params p{};
  int ntotal = 0, ntotal2 = 0, npoints = 1;
  bool dummy_nodes = false;
  double sml = 1.2;
  // module state that time_integration starts from
  std::vector<double> x, vel, stress, mass, rho, hsml, intvars1, f_drucker, x00;
  std::vector<int32_t> itype, bc_or_not, bc_info;
  std::vector<float> wall_position, horizontal_or_not;
  // tables referenced by p
  std::vector<int32_t> nptstcurves;
  std::vector<double> ttcurves, bc_list, segment_bcs, nodal_bcs;
  std::vector<float> ftcurves;
  std::vector<sph_run_block> blocks;
  // output flags of problem_input_data (3_SPH_material_2018.f90:333-336): stress_out(1:4),
  // vel_out(1:2), strain_out, rho_out, sml_out, disp_out
  int32_t out_flags[10] = {1, 1, 1, 1, 1, 1, 1, 0, 0, 0};
  bool gid_started = false;
  // node lattice of the rectangle generator (ndivx columns of ndivy nodes), for the GiD
  // elements of OutputMesh; 0 when the nodes came from elsewhere
  int ndivx = 0, ndivy = 0;
  void fix_pointers() {
    p.nptstcurves = nptstcurves.empty() ? nullptr : nptstcurves.data();
    p.ttcurves = ttcurves.empty() ? nullptr : ttcurves.data();
    p.ftcurves = ftcurves.empty() ? nullptr : ftcurves.data();
    p.bc_list = bc_list.empty() ? nullptr : bc_list.data();
    p.wall_position = wall_position.data();
    p.horizontal_or_not = horizontal_or_not.data();
  }
};

namespace {

struct Wall {
  int id;
  float position, x1, x2;
};

// Read_2DMesh particle generation for the rectangle (3_SPH_material_2018.f90:426-751) and
// set_up_dummy_nodes (:755-897); fills the particle arrays of P in reference order.
void build_rectangle(sph_problem& P, double x1, double x4, double y1, double y4, double dx,
                     double dy, bool inside, int npoints, double rx_factor, double ry_factor,
                     const std::vector<Wall>& walls) {
  const double* props = P.p.props;
  double lx = x4 - x1, ly = y4 - y1;
  int ndivx = (int)(lx / dx + 1.0);
  int ndivy = (int)(ly / dy + 1.0);
  int nnode = ndivx * ndivy;
  P.ndivx = ndivx;
  P.ndivy = ndivy;
  int nstress;
  if (inside) nstress = npoints * (ndivx - 1) * (ndivy - 1);
  else nstress = npoints * nnode;
  int ntotal = nnode + nstress;
  // dummies
  int ndummy2 = 0, ndummy = 0;
  const int nrow = 3;
  float dx2 = (float)dx, dy2 = (float)dy;
  std::vector<int> ndiv_wall;
  if (P.dummy_nodes) {
    for (const Wall& w : walls) {
      float l_wall = w.x2 - w.x1;
      int nd = (int)(l_wall / dx2 + 1.0f);
      ndiv_wall.push_back(nd);
      ndummy2 += nd;
    }
    ndummy = nrow * ndummy2;
  }
  int ntotal2 = ntotal + ndummy;
  P.ntotal = ntotal;
  P.ntotal2 = ntotal2;
  P.p.nnode = nnode;
  P.p.nstress = nstress;
  P.p.ndummy = ndummy;
  P.p.ndummy2 = ndummy2;
  P.x.assign(2 * (size_t)ntotal2, 0.0);
  P.vel.assign(2 * (size_t)ntotal2, 0.0);
  P.stress.assign(4 * (size_t)ntotal2, 0.0);
  P.mass.assign(ntotal2, 0.0);
  P.rho.assign(ntotal2, 0.0);
  P.hsml.assign(ntotal2, 0.0);
  P.itype.assign(ntotal2, 0);
  P.wall_position.assign(ntotal2, 0.0f);
  P.horizontal_or_not.assign(ntotal2, 0.0f);
  // nodes
  std::vector<int> no_int_node(nnode);
  int k = 0;
  for (int i = 1; i <= ndivx; i++)
    for (int j = 1; j <= ndivy; j++) {
      double xx = x1 + (double)(i - 1) * dx;
      double yy = y1 + (double)(j - 1) * dy;
      P.x[2 * k] = xx;
      P.x[2 * k + 1] = yy;
      if (xx == x1 || xx == x4 || yy == y4) no_int_node[k] = 4;
      else no_int_node[k] = 8;
      if ((xx == x1 && (yy == y1 || yy == y4)) || (xx == x4 && (yy == y1 || yy == y4)))
        no_int_node[k] = 2;
      k++;
    }
  auto X1 = [&](int n, int d) { return P.x[2 * (size_t)(n - 1) + d]; };  // x_1(d+1, n)
  // stress points
  std::vector<double> xs(2 * (size_t)nstress);
  if (inside) {
    k = 0;
    if (npoints == 1) {
      for (int i = 2; i <= ndivx; i++)
        for (int j = 2; j <= ndivy; j++) {
          xs[2 * k] = (x1 - dx / 2.0) + (double)(i - 1) * dx;
          xs[2 * k + 1] = (y1 - dx / 2.0) + (double)(j - 1) * dy;
          k++;
        }
    } else if (npoints == 2) {
      for (int j = 1; j <= ndivx - 1; j++)
        for (int i = 1; i <= ndivy - 1; i++) {
          int b = (j - 1) * ndivy;
          xs[2 * k] = ((X1(i + b, 0) + X1(i + 1 + b, 0)) + X1(i + ndivy + b, 0)) / 3.0;
          xs[2 * k + 1] = ((X1(i, 1) + X1(i + 1, 1)) + X1(i + ndivy, 1)) / 3.0;
          xs[2 * k + 2] = ((X1(i + 1 + b, 0) + X1(i + ndivy + b, 0)) + X1(i + ndivy + b, 0)) / 3.0;
          xs[2 * k + 3] = ((X1(i + 1, 1) + X1(i + ndivy, 1)) + X1(i + ndivy + 1, 1)) / 3.0;
          k += 2;
        }
    } else if (npoints == 3) {
      for (int j = 1; j <= ndivx - 1; j++)
        for (int i = 1; i <= ndivy - 1; i++) {
          int b = (j - 1) * ndivy;
          xs[2 * k] = ((X1(i + b, 0) + X1(i + 1 + b, 0)) + X1(i + ndivy + b, 0)) / 3.0;
          xs[2 * k + 1] = ((X1(i, 1) + X1(i + 1, 1)) + X1(i + ndivy, 1)) / 3.0;
          xs[2 * k + 2] = ((X1(i + b, 0) + X1(i + ndivy + b, 0)) + X1(i + 1 + ndivy + b, 0)) / 3.0;
          xs[2 * k + 3] = ((X1(i, 1) + X1(i + ndivy, 1)) + X1(i + ndivy + 1, 1)) / 3.0;
          xs[2 * k + 4] = ((X1(i + 1 + b, 0) + X1(i + 1 + ndivy + b, 0)) +
                           (X1(i + ndivy + b, 0) + X1(i + b, 0)) / 2.0) /
                          3.0;
          xs[2 * k + 5] = ((X1(i + 1, 1) + X1(i + 1 + ndivy, 1)) + (X1(i, 1) + X1(i + 1, 1)) / 2.0) / 3.0;
          k += 3;
        }
    } else if (npoints == 4) {
      for (int j = 1; j <= ndivx - 1; j++)
        for (int i = 1; i <= ndivy - 1; i++) {
          int b = (j - 1) * ndivy;
          xs[2 * k] = ((X1(i + b, 0) + X1(i + b, 0)) + X1(i + 1 + ndivy + b, 0)) / 3.0;
          xs[2 * k + 1] = ((X1(i, 1) + X1(i + 1, 1)) + X1(i + ndivy, 1)) / 3.0;
          xs[2 * k + 2] = ((X1(i + 1 + b, 0) + X1(i + ndivy + b, 0)) + X1(i + ndivy + 1 + b, 0)) / 3.0;
          xs[2 * k + 3] = ((X1(i + 1, 1) + X1(i + ndivy, 1)) + X1(i + ndivy + 1, 1)) / 3.0;
          xs[2 * k + 4] = ((X1(i + b, 0) + X1(i + 1 + b, 0)) + X1(i + 1 + ndivy + b, 0)) / 3.0;
          xs[2 * k + 5] = ((X1(i, 1) + X1(i + 1, 1)) + X1(i + 1 + ndivy, 1)) / 3.0;
          xs[2 * k + 6] = ((X1(i + b, 0) + X1(i + ndivy + b, 0)) + X1(i + 1 + ndivy + b, 0)) / 3.0;
          xs[2 * k + 7] = ((X1(i, 1) + X1(i + ndivy, 1)) + X1(i + ndivy + 1, 1)) / 3.0;
          k += 4;
        }
    }
  } else {
    double r_x = dx * rx_factor, r_y = dx * ry_factor;
    k = 0;
    for (int i = 1; i <= nnode; i++) {
      double nx = X1(i, 0), ny = X1(i, 1);
      if (npoints == 1) {
        xs[2 * k] = nx + r_x;
        xs[2 * k + 1] = ny + r_y;
      } else if (npoints == 2) {
        xs[2 * k] = nx + r_x;
        xs[2 * k + 1] = ny + r_y;
        xs[2 * k + 2] = nx - r_x;
        xs[2 * k + 3] = ny - r_y;
      } else if (npoints == 3) {
        xs[2 * k] = nx;
        xs[2 * k + 1] = ny + r_y;
        xs[2 * k + 2] = nx - r_x;
        xs[2 * k + 3] = ny - r_y;
        xs[2 * k + 4] = nx + r_x;
        xs[2 * k + 5] = ny - r_y;
      } else {
        xs[2 * k] = nx - r_x;
        xs[2 * k + 1] = ny - r_y;
        xs[2 * k + 2] = nx - r_x;
        xs[2 * k + 3] = ny + r_y;
        xs[2 * k + 4] = nx + r_x;
        xs[2 * k + 5] = ny + r_y;
        xs[2 * k + 6] = nx + r_x;
        xs[2 * k + 7] = ny - r_y;
      }
      k += npoints;
    }
  }
  // density, smoothing length, mass (:682-729)
  const double rho0 = props[5];
  for (int i = 0; i < nnode; i++) {
    double area = ((rho0 * dx) * dy) / 8.0;
    P.rho[i] = rho0;
    P.hsml[i] = P.sml * dx;
    P.mass[i] = (double)no_int_node[i] * area;
    P.itype[i] = 2;
  }
  for (int s = 0; s < nstress; s++) {
    int id = nnode + s;
    double area = ((rho0 * dx) * dy) / 8.0;
    P.x[2 * (size_t)id] = xs[2 * (size_t)s];
    P.x[2 * (size_t)id + 1] = xs[2 * (size_t)s + 1];
    P.rho[id] = rho0;
    P.hsml[id] = P.sml * dx;
    P.itype[id] = 1;
    if (inside) P.mass[id] = (8.0 * area) / (double)npoints;
    else P.mass[id] = P.mass[s / npoints] / (double)npoints;
  }
  if (P.dummy_nodes) {
    // innermost layer first (:819-837), then the outer rows (:841-859)
    int l = ntotal;
    auto put = [&](const Wall& w, int j, int m) {
      float xx, yy;
      if (w.id == 1 || w.id == 3) {
        xx = w.position - (float)(m - 1) * dx2;
        yy = w.x1 + (float)(j - 1) * dy2;
        P.horizontal_or_not[l] = (w.id == 1) ? 2.0f : 22.0f;
      } else {
        xx = w.x1 + (float)(j - 1) * dx2;
        yy = w.position - (float)(m - 1) * dy2;
        P.horizontal_or_not[l] = 1.0f;
      }
      P.x[2 * (size_t)l] = (double)xx;
      P.x[2 * (size_t)l + 1] = (double)yy;
      P.wall_position[l] = w.position;
      P.rho[l] = rho0;
      P.mass[l] = (double)(dx2 * dx2) * rho0;
      P.hsml[l] = P.sml * dx;
      P.itype[l] = 25;
      l++;
    };
    for (size_t w = 0; w < walls.size(); w++)
      for (int j = 1; j <= ndiv_wall[w]; j++) put(walls[w], j, 1);
    for (size_t w = 0; w < walls.size(); w++)
      for (int m = 2; m <= nrow; m++)
        for (int j = 1; j <= ndiv_wall[w]; j++) put(walls[w], j, m);
  }
  // elastic constants (:738-749)
  double young = props[2], poiss = props[3];
  double K_mod = young / (3.0 * (1.0 - 2.0 * poiss));
  double G_mod = young / (2.0 * (1.0 + poiss));
  P.p.D11 = (double)(4.0f / 3.0f) * G_mod + K_mod;
  P.p.D22 = P.p.D11;
  P.p.D12 = -((double)(2.0f / 3.0f) * G_mod) + K_mod;
  P.p.D33 = G_mod;
  P.p.D41 = P.p.D12;
  P.p.D42 = P.p.D12;
  P.p.dx = dx;
  P.p.dy = dy;
  P.intvars1.assign(ntotal, 0.0);
  P.f_drucker.assign(ntotal, 0.0);
  P.bc_or_not.assign(ntotal, 0);
  P.bc_info.assign(8 * (size_t)ntotal, 0);
  for (int i = 0; i < ntotal; i++) P.bc_info[8 * (size_t)i] = i + 1;
}

void defaults(sph_problem& P) {
  P.p.ndimn = 2;
  P.p.nstre = 4;
  P.p.pi = (double)(4.0f * std::atan(1.0f));
  P.p.precision = SPS_PREC_FP64_PLAIN;
  // the Drucker-Prager example's copy (the header with ntype_solid): CSPM determinant
  // threshold 1e-07 (2_SPH_main_2018.f90:599), Normal_BCs over nodes and stress-points
  // (3_SPH_material_2018.f90:1683)
  P.p.cspm_det_min = (double)1e-07f;
  P.p.bc_nodes_only = 0;
}

void parse_all(sph_problem& P, const std::string& in_txt, const std::string& dat_txt,
               const std::string& pts_txt) {
  ListReader in(in_txt, "input.txt"), dat(dat_txt, ".dat"), pts(pts_txt, ".pts");
  defaults(P);
  in.text();
  P.name = in.read(1)[0];
  // problem_input_data (:64-163)
  int nline = dat.integer();
  for (int i = 0; i < nline; i++) dat.text();
  dat.text();
  P.p.ndimn = dat.integer();
  if (P.p.ndimn != 2) throw ParseError("only ndimn = 2 is supported");
  dat.text();
  int ntype_solid = 0, nstre, nmats;
  if (dat.peek_count() >= 3) {
    auto v = dat.read(3);
    ntype_solid = dat.to_i(v[0]);
    nstre = dat.to_i(v[1]);
    nmats = dat.to_i(v[2]);
  } else {
    // the header of code/ and of the strain-localisation and vertical-slope copies
    // (`nstre, nmats`, code/3_SPH_material_2018.f90:101).  The strain-localisation copy's
    // constitutive routines are the plane-strain branch without a test ("nstre = 4 --
    // plane strain (only current functioning option)"), i.e. ntype_solid 2 here; the
    // vertical-slope copy never reads ntype_solid (0), which its elastic example reaches
    // no branch of.  The CSPM threshold of all three is 1e-03 (2_SPH_main_2018.f90:599);
    // code/ and the strain-localisation copy apply Normal_BCs to the nodes only
    // (3_SPH_material_2018.f90:1664), the vertical-slope copy to 1..ntotal: a caller
    // replacing that copy sets bc_nodes_only = 0.
    auto v = dat.read(2);
    nstre = dat.to_i(v[0]);
    nmats = dat.to_i(v[1]);
    ntype_solid = 2;
    P.p.cspm_det_min = (double)1e-03f;
    P.p.bc_nodes_only = 1;
  }
  P.p.ntype_solid = ntype_solid;
  if (ntype_solid == 4) nstre = 6;
  P.p.nstre = nstre;
  if (nstre != 4) throw ParseError("only nstre = 4 is supported");
  dat.text();
  for (int m = 0; m < nmats; m++) {
    auto v = dat.read(13);
    int lmat = dat.to_i(v[0]);
    double props[20] = {0};
    for (int k = 0; k < 12; k++) props[k] = dat.to_d(v[1 + k]);
    int ncrit = (int)props[1];
    if (ncrit == 5 || ncrit == 12) {
      dat.text();
      auto w = dat.read(8);
      for (int k = 0; k < 8; k++) props[12 + k] = dat.to_d(w[k]);
    }
    if (lmat == 1) std::memcpy(P.p.props, props, sizeof(props));
  }
  // setup_particles (:344-360) -> Read_2DMesh (:365)
  dat.text();
  dat.integer();
  in.text();
  auto f3 = in.read(3);
  bool sp_sph = in.to_l(f3[0]);
  bool art_stress = in.to_l(f3[1]);
  bool inside = false, vel_vector = false, sph_shift = false;
  int npoints = 1, shift_update = 1;
  double rx = 0, ry = 0, disp_tol = 0;
  if (sp_sph) {
    in.text();
    inside = in.logical();
    in.text();
    npoints = in.integer();
    if (!inside) {
      in.text();
      auto v = in.read(6);
      sph_shift = in.to_l(v[0]);
      vel_vector = in.to_l(v[1]);
      shift_update = in.to_i(v[2]);
      rx = in.to_d(v[3]);
      ry = in.to_d(v[4]);
      disp_tol = in.to_d(v[5]);
    }
  }
  if (vel_vector) npoints = 2;
  if (!sp_sph) npoints = 1;
  P.npoints = npoints;
  P.p.npoints = npoints;
  P.p.sph_shift = sph_shift;
  P.p.vel_vector = vel_vector;
  P.p.shift_update = shift_update;
  P.p.disp_tol = disp_tol;
  pts.text();
  pts.integer();  // geom_type: always a rectangle in the reference
  pts.text();
  auto xv = pts.read(5);
  pts.text();
  auto yv = pts.read(5);
  pts.text();
  P.dummy_nodes = pts.logical();
  double x1 = pts.to_d(xv[0]), x4 = pts.to_d(xv[3]), dx = pts.to_d(xv[4]);
  double y1 = pts.to_d(yv[0]), y4 = pts.to_d(yv[3]), dy = pts.to_d(yv[4]);
  in.text();
  P.sml = in.dbl();
  std::vector<Wall> walls;
  if (P.dummy_nodes) {
    pts.text();
    int n_walls = pts.integer();
    for (int i = 0; i < n_walls; i++) {
      pts.text();
      pts.text();
      auto v = pts.read(4);
      walls.push_back({pts.to_i(v[0]), pts.to_f(v[1]), pts.to_f(v[2]), pts.to_f(v[3])});
    }
  }
  P.p.sp_sph = sp_sph;
  P.p.inside_approach = inside;
  P.p.art_stress = art_stress;
  P.p.r_x = dx * rx;  // Read_2DMesh (:628)
  P.p.r_y = dx * ry;
  if (!sp_sph) {
    // Standard SPH: stress-points coincide with nodes (outside approach with zero shift)
    build_rectangle(P, x1, x4, y1, y4, dx, dy, false, 1, 0.0, 0.0, walls);
  } else {
    build_rectangle(P, x1, x4, y1, y4, dx, dy, inside, npoints, rx, ry, walls);
  }
  // boundary conditions (:182-231)
  dat.text();
  auto b2 = dat.read(2);
  P.p.no_bcs = dat.to_i(b2[0]);
  P.p.ifsigman = dat.to_i(b2[1]);
  if (P.p.no_bcs > 0) {
    float twopi = std::acos(0.0f) * 4.0f / 360.0f;
    dat.text();
    P.bc_list.assign(8 * (size_t)P.p.no_bcs, 0.0);
    for (int i = 0; i < P.p.no_bcs; i++) {
      auto v = dat.read(8);
      for (int j = 0; j < 8; j++) P.bc_list[j + 8 * (size_t)i] = dat.to_d(v[j]);
      P.bc_list[6 + 8 * (size_t)i] = P.bc_list[6 + 8 * (size_t)i] * (double)twopi;
    }
  }
  dat.text();
  int nseg = dat.integer();
  if (nseg > 0) {
    dat.text();
    for (int i = 0; i < nseg; i++) {
      auto v = dat.read(5);
      for (int j = 0; j < 5; j++) P.segment_bcs.push_back(dat.to_d(v[j]));
    }
  }
  dat.text();
  int nnod = dat.integer();
  if (nnod > 0) {
    dat.text();
    for (int i = 0; i < nnod; i++) {
      auto v = dat.read(2);
      for (int j = 0; j < 2; j++) P.nodal_bcs.push_back(dat.to_d(v[j]));
    }
  }
  // Get_BCs_on_node (:1049-1131)
  for (int s = 0; s < nseg; s++) {
    const double* g = &P.segment_bcs[5 * (size_t)s];
    double xx1 = g[0], yy1 = g[1], xx2 = g[2], yy2 = g[3];
    double xmax = std::max(xx1, xx2), xmin = std::min(xx1, xx2);
    double ymax = std::max(yy1, yy2), ymin = std::min(yy1, yy2);
    int no_bc = (int)g[4];
    for (int ip = 0; ip < P.ntotal; ip++) {
      double xx = P.x[2 * (size_t)ip], yy = P.x[2 * (size_t)ip + 1];
      double z = (yy1 - yy2) * (xx - xx1) + (xx2 - xx1) * (yy - yy1);
      if (z == 0.0 && xx >= xmin && xx <= xmax && yy >= ymin && yy <= ymax) {
        int kk = ++P.bc_info[1 + 8 * (size_t)ip];
        if (kk + 2 > 8) throw ParseError("more than 6 boundary conditions on one particle");
        P.bc_info[kk + 1 + 8 * (size_t)ip] = no_bc;
        if (P.bc_or_not[ip] == 0) P.bc_or_not[ip] = 1;
      }
    }
  }
  for (int s = 0; s < nnod; s++) {
    int ic_node = (int)P.nodal_bcs[2 * (size_t)s];
    int no_bc = (int)P.nodal_bcs[2 * (size_t)s + 1];
    if (ic_node < 1 || ic_node > P.ntotal || no_bc < 1 || no_bc > P.p.no_bcs)
      throw ParseError("nodal boundary condition out of range");
    int bc_var = (int)P.bc_list[1 + 8 * (size_t)(no_bc - 1)];
    int32_t* bi = &P.bc_info[8 * (size_t)(ic_node - 1)];
    bi[1]++;
    int kk = bc_var + 2;
    if (kk < 1 || kk > 8) throw ParseError("nodal boundary condition variable out of range");
    if (bi[kk - 1] != 0 && bi[kk - 1] != no_bc)
      // the reference asks on stdin which one to keep (:1117-1122); a batch reader cannot
      throw ParseError("conflicting nodal boundary conditions on one node");
    bi[kk - 1] = no_bc;
    if (P.bc_or_not[ic_node - 1] == 0) P.bc_or_not[ic_node - 1] = 1;
  }
  // time curves (:234-264)
  dat.text();
  int ic_tcurve = dat.integer();
  if (ic_tcurve == 1) {
    dat.text();
    auto v = dat.read(2);
    int nt = dat.to_i(v[0]), mp = dat.to_i(v[1]);
    P.p.ntcurves = nt;
    P.p.mptstcurves = mp;
    P.nptstcurves.assign(nt, 0);
    P.ttcurves.assign((size_t)nt * mp, 0.0);
    P.ftcurves.assign((size_t)nt * mp, 0.0f);
    for (int i = 0; i < nt; i++) {
      dat.text();
      int np = dat.integer();
      if (np > mp) throw ParseError("time curve longer than its declared maximum");
      P.nptstcurves[i] = np;
      dat.text();
      auto tv = dat.read(np);
      auto fv = dat.read(np);
      for (int j = 0; j < np; j++) {
        P.ttcurves[i + (size_t)j * nt] = dat.to_d(tv[j]);
        P.ftcurves[i + (size_t)j * nt] = dat.to_f(fv[j]);
      }
    }
  }
  dat.text();
  auto dom = dat.read(4);
  P.p.xmin_domain[0] = dat.to_d(dom[0]);
  P.p.xmin_domain[1] = dat.to_d(dom[1]);
  P.p.xmax_domain[0] = dat.to_d(dom[2]);
  P.p.xmax_domain[1] = dat.to_d(dom[3]);
  // Initial_conditions (:1433-1569)
  dat.text();
  int icunkno = dat.integer();
  if (icunkno == 2) {
    for (int k = 0; k < nstre + 2; k++) {
      dat.text();
      dat.integer();
    }
  } else if (icunkno == 30) {
    dat.text();
    int type_sigma0 = dat.integer();
    if (type_sigma0 == 1) {
      dat.text();
      auto sv = dat.read(nstre);
      dat.text();
      auto iv = dat.read(10);
      for (int ip = 0; ip < P.ntotal; ip++) {
        for (int a = 0; a < 4; a++) P.stress[a + 4 * (size_t)ip] = dat.to_d(sv[a]);
        P.intvars1[ip] = dat.to_d(iv[0]);
      }
    }
  }
  // control parameters (:302-336)
  dat.text();
  auto cv = dat.read(7);
  P.p.sle = dat.to_i(cv[2]);
  P.p.skf = dat.to_i(cv[3]);
  P.p.cspm = dat.to_l(cv[4]);
  P.p.update_x = dat.to_l(cv[5]);
  P.p.xsph = dat.to_l(cv[6]);
  dat.text();
  auto dv = dat.read(2);
  P.p.cont_density = dat.to_l(dv[1]);
  dat.text();
  P.p.damping = dat.dbl();
  dat.text();
  auto ab = dat.read(2);
  P.p.alpha = dat.to_d(ab[0]);
  P.p.beta = dat.to_d(ab[1]);
  dat.text();
  P.p.ic_grav = dat.integer();
  if (P.p.ic_grav == 1) {
    dat.text();
    auto g = dat.read(4);
    P.p.cgrav[0] = dat.to_d(g[0]);
    P.p.cgrav[1] = dat.to_d(g[1]);
    P.p.tcurve_grav = dat.to_i(g[2]);
    P.p.ft_grav = dat.to_d(g[3]);
  }
  dat.text();
  dat.text();
  {
    auto of = dat.read(10);
    for (int k = 0; k < 10; k++) P.out_flags[k] = dat.to_i(of[k]);
  }
  // driver time blocks (code/1_SPH_2018.f90:50-106)
  for (;;) {
    in.text();
    auto t = in.read(3);
    sph_run_block b{};
    b.dt = in.to_d(t[0]);
    b.time_end = in.to_d(t[1]);
    b.maxtimestep = in.to_i(t[2]);
    if (b.dt <= 0) break;
    in.text();
    auto o = in.read(3);
    b.print_step = in.to_i(o[0]);
    b.save_step = in.to_i(o[1]);
    b.plot_step = in.to_i(o[2]);
    P.blocks.push_back(b);
  }
  if (!P.blocks.empty()) P.p.dt_sph = P.blocks[0].dt;
  P.x00 = P.x;
  P.fix_pointers();
}

std::string slurp(const std::string& path) {
  std::ifstream f(path);
  if (!f) throw ParseError("cannot open " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  return ss.str();
}

void set_err(char* err, int32_t len, const std::string& m) {
  if (err && len > 0) {
    std::snprintf(err, (size_t)len, "%s", m.c_str());
  }
}

std::string fmt(const char* f, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, f);
  std::vsnprintf(buf, sizeof buf, f, ap);
  va_end(ap);
  return buf;
}

}  // namespace

extern "C" {

int sph_problem_parse(const char* input_txt, const char* dat, const char* pts, sph_problem** out,
                      char* err, int32_t errlen) {
  if (!input_txt || !dat || !pts || !out) return SPS_ERR_ARG;
  *out = nullptr;
  auto P = std::make_unique<sph_problem>();
  try {
    parse_all(*P, input_txt, dat, pts);
  } catch (const std::exception& e) {
    set_err(err, errlen, e.what());
    return SPS_ERR_ARG;
  }
  *out = P.release();
  return SPS_OK;
}

int sph_problem_read(const char* dir, sph_problem** out, char* err, int32_t errlen) {
  if (!dir || !out) return SPS_ERR_ARG;
  *out = nullptr;
  try {
    std::string d(dir);
    std::string in = slurp(d + "/input.txt");
    ListReader r(in, "input.txt");
    r.text();
    std::string name = r.read(1)[0];
    std::string dat = slurp(d + "/" + name + ".dat");
    std::string pts = slurp(d + "/" + name + ".pts");
    return sph_problem_parse(in.c_str(), dat.c_str(), pts.c_str(), out, err, errlen);
  } catch (const std::exception& e) {
    set_err(err, errlen, e.what());
    return SPS_ERR_ARG;
  }
}

int sph_problem_column(const sph_column_spec* s, sph_problem** out) {
  if (!s || !out || s->dx <= 0 || s->width <= 0 || s->height <= 0) return SPS_ERR_ARG;
  *out = nullptr;
  const double h = s->sml * s->dx;
  double dt = s->dt > 0 ? s->dt : 0.1 * h / std::sqrt(s->young / s->rho);
  const double tanphi = std::tan(s->phi_deg * M_PI / 180.0);
  std::string pts = "geom_type\n1\nx1 x2 x3 x4 dx\n" +
                    fmt("0 %.17g 0 %.17g %.17g\n", s->width, s->width, s->dx) +
                    "y1 y2 y3 y4 dy\n" +
                    fmt("0 0 %.17g %.17g %.17g\n", s->height, s->height, s->dx) +
                    "dummy_nodes\nT\nnumber_of_walls\n2\nwall_1 - LHS wall\nid position x1 x2\n" +
                    fmt("1 %.9g %.9g %.9g\n", -s->dx, -3 * s->dx, s->height + 3 * s->dx) +
                    "wall_2 - bottom wall\nid position x1 x2\n" +
                    fmt("2 %.9g %.9g %.9g\n", -s->dx, -3 * s->dx, s->floor_length);
  std::string dat =
      "1\ngranular column collapse\nndimn\n2\nntype_solid nstre nmats\n2 4 1\n"
      "mater. eco law E Poiss b rho yield H ? gamma delta n\n" +
      fmt("1 2 12 %.17g %.17g 1. %.17g 2000. 0 0. 5. 1. 1\n", s->young, s->poiss, s->rho) +
      "tan(phi) cohesion\n" + fmt("%.17g %.17g 0 0 0 0 0 0\n", tanphi, s->cohesion) +
      "ic_unks\n0\nBC's\n0 0\nsegments\n0\nnodes\n0\nic_tcurve\n1\ncurves\n1 100\npts\n3\n"
      "times_and_factors\n0 1 1e9\n1 1 1\ndomain\n-1e6 -1e6 1e6 1e6\nIC\n2\n"
      "s11\n0\ns22\n0\ns12\n0\ns33\n0\nw1\n0\nv2\n0\n"
      "pa_sph nnps sle skf cspm update_x XSPH\n" +
      fmt("2 2 1 1 %s T %s\n", s->cspm ? "T" : "F", s->xsph ? "T" : "F") +
      "summ cont\nF F\ndamping\n" + fmt("%.17g\n", s->damping) + "alpha beta\n" +
      fmt("%.17g %.17g\n", s->alpha, s->beta) +
      "ic_grav\n1\ngx gy timecurve factor\n0 -9.81 1 1.\noutput\n"
      "sxx syy sxy szz vx vy strain rho sml disp\n1 1 1 1 1 1 1 0 0 0\n";
  std::string in = "problem name\ncolumn\nSP_SPH art_stress particle_shift\nT F F\n"
                   "inside_approach\nT\nnpoints\n1\nsml\n" +
                   fmt("%.17g\n", s->sml) + "dt\n" + fmt("%.17g,1e9,1000000000\n", dt) +
                   "print save plot\n1000000000,1000000000,1000000000\nend\n-1,1,1\n";
  sph_problem* P = nullptr;
  int rc = sph_problem_parse(in.c_str(), dat.c_str(), pts.c_str(), &P, nullptr, 0);
  if (rc) return rc;
  // K0 geostatic stress (extension of the reference's zero/constant initial conditions)
  const double g = 9.81;
  for (int ip = 0; ip < P->ntotal; ip++) {
    double depth = s->height - P->x[2 * (size_t)ip + 1];
    if (depth < 0) depth = 0;
    double syy = -s->rho * g * depth;
    P->stress[0 + 4 * (size_t)ip] = s->k0 * syy;
    P->stress[1 + 4 * (size_t)ip] = syy;
    P->stress[2 + 4 * (size_t)ip] = 0.0;
    P->stress[3 + 4 * (size_t)ip] = s->k0 * syy;
  }
  *out = P;
  return SPS_OK;
}

int sph_problem_biaxial(const sph_biaxial_spec* s, sph_problem** out) {
  if (!s || !out || s->dx <= 0 || s->width <= 0 || s->height <= 0 || s->confining < 0 ||
      s->q_ratio < 0 || s->q_ratio >= 1 || s->t_ramp <= 0)
    return SPS_ERR_ARG;
  *out = nullptr;
  const double h = s->sml * s->dx;
  const double dt = s->dt > 0 ? s->dt : 0.1 * h / std::sqrt(s->young / s->rho);
  const double tanphi = std::tan(s->phi_deg * M_PI / 180.0);
  std::string pts = "geom_type\n1\nx1 x2 x3 x4 dx\n" +
                    fmt("0 %.17g 0 %.17g %.17g\n", s->width, s->width, s->dx) +
                    "y1 y2 y3 y4 dy\n" +
                    fmt("0 0 %.17g %.17g %.17g\n", s->height, s->height, s->dx) +
                    "dummy_nodes\nF\n";
  std::string in = "problem name\nbiaxial\nSP_SPH art_stress particle_shift\nT F F\n"
                   "inside_approach\nT\nnpoints\n1\nsml\n" +
                   fmt("%.17g\n", s->sml) + "dt\n" + fmt("%.17g,1e9,1000000000\n", dt) +
                   "print save plot\n1000000000,1000000000,1000000000\nend\n-1,1,1\n";
  auto dat_text = [&](double xr, double yt) {
    // BCs of Normal_BCs (3_SPH_material_2018.f90:1666-1773): var 5 = vx, 6 = vy, 1 = sxx,
    // 3 = sxy; curve 1 ramps the platen velocity in over t_ramp, curve 2 holds the
    // confining stress.  The segments lie on the outermost node rows and columns (their
    // coordinates as generated), which Get_BCs_on_node's exact collinearity test needs.
    std::string bcs = "BC's\n5 0\nnber var t_variation a1 a0 w fi Tf\n" +
                      fmt("1 5 1 0 0 0 0 0\n2 6 1 %.17g 0 0 0 0\n3 6 1 %.17g 0 0 0 0\n",
                          -s->platen_v, s->platen_v) +
                      fmt("4 1 2 %.17g 0 0 0 0\n5 3 2 0 0 0 0 0\n", -s->confining) +
                      "segments\n8\nx1 y1 x2 y2 bc\n" +
                      fmt("0 %.17g %.17g %.17g 1\n0 %.17g %.17g %.17g 2\n", yt, xr, yt, yt, xr,
                          yt) +
                      fmt("0 0 %.17g 0 1\n0 0 %.17g 0 3\n", xr, xr) +
                      fmt("0 0 0 %.17g 4\n0 0 0 %.17g 5\n", yt, yt) +
                      fmt("%.17g 0 %.17g %.17g 4\n%.17g 0 %.17g %.17g 5\n", xr, xr, yt, xr, xr,
                          yt);
    return "1\nbiaxial compression\nndimn\n2\nntype_solid nstre nmats\n2 4 1\n"
           "mater. eco law E Poiss b rho yield H ? gamma delta n\n" +
           fmt("1 2 12 %.17g %.17g 1. %.17g 2000. 0 0. 5. 1. 1\n", s->young, s->poiss,
               s->rho) +
           "tan(phi) cohesion\n" + fmt("%.17g %.17g 0 0 0 0 0 0\n", tanphi, s->cohesion) +
           "ic_unks\n0\n" + bcs + "nodes\n0\nic_tcurve\n1\ncurves\n2 100\npts\n3\ntimes\n" +
           fmt("0 %.17g 1e9\n0 1 1\n", s->t_ramp) + "pts\n2\ntimes\n0 1e9\n1 1\n" +
           "domain\n-1e6 -1e6 1e6 1e6\nIC\n2\n"
           "s11\n0\ns22\n0\ns12\n0\ns33\n0\nw1\n0\nv2\n0\n"
           "pa_sph nnps sle skf cspm update_x XSPH\n2 2 1 1 F T F\n"
           "summ cont\nF F\ndamping\n0\nalpha beta\n0 0\nic_grav\n0\noutput\n"
           "sxx syy sxy szz vx vy strain rho sml disp\n1 1 1 1 1 1 1 0 0 0\n";
  };
  // the node lattice as generated: its last column and row carry the platen and side BCs
  sph_problem* P0 = nullptr;
  int rc = sph_problem_parse(in.c_str(), dat_text(s->width, s->height).c_str(), pts.c_str(),
                             &P0, nullptr, 0);
  if (rc) return rc;
  double xr = 0.0, yt = 0.0;
  for (int ip = 0; ip < P0->p.nnode; ip++) {
    xr = std::max(xr, P0->x[2 * (size_t)ip]);
    yt = std::max(yt, P0->x[2 * (size_t)ip + 1]);
  }
  sph_problem_free(P0);
  sph_problem* P = nullptr;
  rc = sph_problem_parse(in.c_str(), dat_text(xr, yt).c_str(), pts.c_str(), &P, nullptr, 0);
  if (rc) return rc;
  // initial stress (an extension of the reference's zero/constant initial conditions):
  // confining pressure p on every face plus an axial excess q_ratio * q_y, where q_y is the
  // axial excess at which the Drucker-Prager function sqrt(J2) + alpha I1 - k_c reaches 0
  // (sxx = szz = -p, syy = -p - q: sqrt(J2) = q / sqrt(3), I1 = -3p - q)
  const double root = std::sqrt(9.0 + 12.0 * tanphi * tanphi);
  const double alpha = tanphi / root, kc = 3.0 * s->cohesion / root;
  const double qy = (3.0 * alpha * s->confining + kc) / (1.0 / std::sqrt(3.0) - alpha);
  const double q = s->q_ratio * qy;
  for (int ip = 0; ip < P->ntotal; ip++) {
    P->stress[0 + 4 * (size_t)ip] = -s->confining;
    P->stress[1 + 4 * (size_t)ip] = -s->confining - q;
    P->stress[2 + 4 * (size_t)ip] = 0.0;
    P->stress[3 + 4 * (size_t)ip] = -s->confining;
  }
  *out = P;
  return SPS_OK;
}

int sph_problem_slope(const sph_slope_spec* s, sph_problem** out) {
  if (!s || !out || s->dx <= 0 || s->Lf <= 0 || s->Hf <= 0 || s->Ls < 0 || s->Hs < 0 ||
      s->Ls > s->Lf)
    return SPS_ERR_ARG;
  *out = nullptr;
  auto P = std::make_unique<sph_problem>();
  defaults(*P);
  sph_problem& Q = *P;
  Q.name = "slope";
  const double dx = s->dx, h = s->sml * dx;
  const double tanphi = std::tan(s->phi_deg * M_PI / 180.0);
  Q.sml = s->sml;
  Q.p.ntype_solid = 2;
  Q.p.props[0] = 2;
  Q.p.props[1] = 12;
  Q.p.props[2] = s->young;
  Q.p.props[3] = s->poiss;
  Q.p.props[4] = 1.0;
  Q.p.props[5] = s->rho;
  Q.p.props[12] = tanphi;
  Q.p.props[13] = s->cohesion;
  Q.p.sp_sph = 1;
  Q.p.inside_approach = 1;
  Q.p.skf = 1;
  Q.p.sle = 1;
  Q.p.update_x = 1;
  Q.p.xsph = s->xsph;
  Q.p.alpha = s->alpha;
  Q.p.beta = s->beta;
  Q.p.damping = s->damping;
  Q.p.dt_sph = s->dt > 0 ? s->dt : 0.1 * h / std::sqrt(s->young / s->rho);
  // lattice: columns i = 0..nfx, rows j = 0..; node present when inside the union
  const int nfx = (int)std::lround(s->Lf / dx), nfy = (int)std::lround(s->Hf / dx);
  const int nsx = (int)std::lround(s->Ls / dx), nsy = (int)std::lround(s->Hs / dx);
  const int ny_tot = nfy + nsy;
  // inclined face: horizontal run per unit height (0 for a vertical face)
  const double cot = (s->face_deg > 0.0 && s->face_deg < 90.0)
                         ? 1.0 / std::tan(s->face_deg * M_PI / 180.0) : 0.0;
  if ((double)nsx + (double)nsy * cot > (double)nfx) return SPS_ERR_ARG;  // toe off the foundation
  auto node_in = [&](int i, int j) {
    if (i < 0 || j < 0 || i > nfx || j > ny_tot) return false;
    if (j <= nfy) return true;
    return (double)i <= (double)nsx + (double)(ny_tot - j) * cot + 1e-9;
  };
  auto cell_in = [&](int i, int j) {  // cell with lower-left node (i,j)
    return node_in(i, j) && node_in(i + 1, j) && node_in(i, j + 1) && node_in(i + 1, j + 1);
  };
  std::vector<int> nid((size_t)(nfx + 1) * (ny_tot + 1), -1);
  int nnode = 0, nstress = 0;
  for (int i = 0; i <= nfx; i++)
    for (int j = 0; j <= ny_tot; j++)
      if (node_in(i, j)) nid[(size_t)i * (ny_tot + 1) + j] = nnode++;
  for (int i = 0; i < nfx; i++)
    for (int j = 0; j < ny_tot; j++)
      if (cell_in(i, j)) nstress++;
  // walls: floor under the foundation, left and right walls of the foundation
  float dx2 = (float)dx;
  std::vector<Wall> walls = {{1, -dx2, -3 * dx2, (float)(s->Hf + 3 * dx)},
                             {2, -dx2, -3 * dx2, (float)(s->Lf + 3 * dx)},
                             {3, (float)(s->Lf + dx), -3 * dx2, (float)(s->Hf + 3 * dx)}};
  std::vector<int> ndiv_wall;
  int ndummy2 = 0;
  for (const Wall& w : walls) {
    int nd = (int)((w.x2 - w.x1) / dx2 + 1.0f);
    ndiv_wall.push_back(nd);
    ndummy2 += nd;
  }
  const int nrow = 3;
  int ndummy = nrow * ndummy2;
  int ntotal = nnode + nstress, ntotal2 = ntotal + ndummy;
  Q.ntotal = ntotal;
  Q.ntotal2 = ntotal2;
  Q.p.nnode = nnode;
  Q.p.nstress = nstress;
  Q.p.ndummy = ndummy;
  Q.p.ndummy2 = ndummy2;
  Q.x.assign(2 * (size_t)ntotal2, 0.0);
  Q.vel.assign(2 * (size_t)ntotal2, 0.0);
  Q.stress.assign(4 * (size_t)ntotal2, 0.0);
  Q.mass.assign(ntotal2, 0.0);
  Q.rho.assign(ntotal2, s->rho);
  Q.hsml.assign(ntotal2, s->sml * dx);
  Q.itype.assign(ntotal2, 0);
  Q.wall_position.assign(ntotal2, 0.0f);
  Q.horizontal_or_not.assign(ntotal2, 0.0f);
  const double area = ((s->rho * dx) * dx) / 8.0;
  for (int i = 0; i <= nfx; i++)
    for (int j = 0; j <= ny_tot; j++) {
      int id = nid[(size_t)i * (ny_tot + 1) + j];
      if (id < 0) continue;
      Q.x[2 * (size_t)id] = (double)i * dx;
      Q.x[2 * (size_t)id + 1] = (double)j * dx;
      int nc = cell_in(i, j) + cell_in(i - 1, j) + cell_in(i, j - 1) + cell_in(i - 1, j - 1);
      Q.mass[id] = (double)(2 * nc) * area;
      Q.itype[id] = 2;
    }
  int sp = nnode;
  for (int i = 0; i < nfx; i++)
    for (int j = 0; j < ny_tot; j++)
      if (cell_in(i, j)) {
        Q.x[2 * (size_t)sp] = ((double)i + 0.5) * dx;
        Q.x[2 * (size_t)sp + 1] = ((double)j + 0.5) * dx;
        Q.mass[sp] = 8.0 * area;
        Q.itype[sp] = 1;
        sp++;
      }
  int l = ntotal;
  auto put = [&](const Wall& w, int j, int m) {
    float xx, yy;
    if (w.id == 1 || w.id == 3) {
      float sgn = (w.id == 1) ? 1.0f : -1.0f;
      xx = w.position - sgn * (float)(m - 1) * dx2;
      yy = w.x1 + (float)(j - 1) * dx2;
      Q.horizontal_or_not[l] = (w.id == 1) ? 2.0f : 22.0f;
    } else {
      xx = w.x1 + (float)(j - 1) * dx2;
      yy = w.position - (float)(m - 1) * dx2;
      Q.horizontal_or_not[l] = 1.0f;
    }
    Q.x[2 * (size_t)l] = (double)xx;
    Q.x[2 * (size_t)l + 1] = (double)yy;
    Q.wall_position[l] = w.position;
    Q.mass[l] = (double)(dx2 * dx2) * s->rho;
    Q.itype[l] = 25;
    l++;
  };
  for (size_t w = 0; w < walls.size(); w++)
    for (int j = 1; j <= ndiv_wall[w]; j++) put(walls[w], j, 1);
  for (size_t w = 0; w < walls.size(); w++)
    for (int m = 2; m <= nrow; m++)
      for (int j = 1; j <= ndiv_wall[w]; j++) put(walls[w], j, m);
  double K_mod = s->young / (3.0 * (1.0 - 2.0 * s->poiss));
  double G_mod = s->young / (2.0 * (1.0 + s->poiss));
  Q.p.D11 = (double)(4.0f / 3.0f) * G_mod + K_mod;
  Q.p.D22 = Q.p.D11;
  Q.p.D12 = -((double)(2.0f / 3.0f) * G_mod) + K_mod;
  Q.p.D33 = G_mod;
  Q.p.D41 = Q.p.D12;
  Q.p.D42 = Q.p.D12;
  Q.p.dx = dx;
  Q.p.dy = dx;
  Q.p.xmin_domain[0] = -1e6;
  Q.p.xmin_domain[1] = -1e6;
  Q.p.xmax_domain[0] = 1e6;
  Q.p.xmax_domain[1] = 1e6;
  // gravity ramp 0 -> 1 over t_ramp
  Q.p.ic_grav = 1;
  Q.p.tcurve_grav = 1;
  Q.p.cgrav[1] = -9.81;
  Q.p.ft_grav = 1.0;
  Q.p.ntcurves = 1;
  Q.p.mptstcurves = 3;
  Q.nptstcurves = {3};
  Q.ttcurves = {0.0, s->t_ramp > 0 ? s->t_ramp : 1e-12, 1e9};
  Q.ftcurves = {s->t_ramp > 0 ? 0.0f : 1.0f, 1.0f, 1.0f};
  // K0 stress of the full gravity load on nodes and stress-points
  const double g = 9.81;
  for (int ip = 0; ip < ntotal; ip++) {
    double xx = Q.x[2 * (size_t)ip], yy = Q.x[2 * (size_t)ip + 1];
    double top = s->Hf;
    if (xx <= s->Ls + 1e-12) top = s->Hf + s->Hs;
    else if (cot > 0.0 && xx < s->Ls + s->Hs * cot) top = s->Hf + s->Hs - (xx - s->Ls) / cot;
    double depth = top - yy;
    if (depth < 0) depth = 0;
    double syy = -s->rho * g * depth;
    Q.stress[0 + 4 * (size_t)ip] = s->k0 * syy;
    Q.stress[1 + 4 * (size_t)ip] = syy;
    Q.stress[3 + 4 * (size_t)ip] = s->k0 * syy;
  }
  Q.intvars1.assign(ntotal, 0.0);
  Q.f_drucker.assign(ntotal, 0.0);
  Q.bc_or_not.assign(ntotal, 0);
  Q.bc_info.assign(8 * (size_t)ntotal, 0);
  for (int i = 0; i < ntotal; i++) Q.bc_info[8 * (size_t)i] = i + 1;
  Q.x00 = Q.x;
  sph_run_block b{};
  b.dt = Q.p.dt_sph;
  b.time_end = 1e9;
  b.maxtimestep = 1000000000;
  b.print_step = b.save_step = b.plot_step = 1000000000;
  Q.blocks.push_back(b);
  Q.fix_pointers();
  *out = P.release();
  return SPS_OK;
}

const sps_params* sph_problem_params(const sph_problem* p) { return p ? &p->p : nullptr; }

int32_t sph_sizeof_params(void) { return (int32_t)sizeof(sps_params); }

int sph_problem_output_flags(const sph_problem* p, int32_t* flags) {
  if (!p || !flags) return SPS_ERR_ARG;
  for (int k = 0; k < 10; k++) flags[k] = p->out_flags[k];
  return SPS_OK;
}

namespace {

// the F16.8 edit descriptor: 16 wide, 8 decimals, 16 asterisks when the value does not fit
void put_f16_8(std::string& o, double v) {
  char b[64];
  int n = std::snprintf(b, sizeof b, "%16.8f", v);
  if (n > 16) o.append(16, '*');
  else o.append(b, (size_t)n);
}

// list-directed output (write(u,*)): a leading blank, then each item; reals with 17
// significant digits.  The spacing of list-directed output is compiler-specific; readers of
// these files split on blanks and commas.
void put_ld_real(std::string& o, double v) {
  char b[64];
  std::snprintf(b, sizeof b, " %24.16E", v);
  o += b;
}
void put_ld_int(std::string& o, long v) {
  char b[32];
  std::snprintf(b, sizeof b, " %11ld", v);
  o += b;
}

bool write_file(const std::string& path, const std::string& text, bool append) {
  FILE* f = std::fopen(path.c_str(), append ? "ab" : "wb");
  if (!f) return false;
  bool ok = std::fwrite(text.data(), 1, text.size(), f) == text.size();
  return std::fclose(f) == 0 && ok;
}

}  // namespace

int sph_write_output(sph_problem* p, const char* dir, int32_t itimestep, double time_sph,
                     const double* x, const double* vel, const double* stress,
                     const double* intvars1, const double* rho, const double* hsml,
                     const int32_t* bc_or_not, const double* displ) {
  if (!p || !dir || !x || !vel || !stress) return SPS_ERR_ARG;
  const int32_t* f = p->out_flags;  // sxx syy sxy szz vx vy strain rho sml disp
  const int nn = p->p.nnode, nt = p->ntotal;
  auto iv = [&](int i) { return intvars1 ? intvars1[i] : 0.0; };
  auto dsp = [&](int i, int k) { return displ ? displ[2 * (size_t)i + k] : 0.0; };
  char suffix[32];
  std::snprintf(suffix, sizeof suffix, "%06d", (int)itimestep);
  const std::string d = std::string(dir) + "/";
  const char* sname[4] = {"sxx", "syy", "sxy", "szz"};
  // nodes.csv: the header and the separators as the reference's node file has them (a comma
  // before each column after the first; its header starts "x-coord,,y-coord")
  std::string o = "x-coord,,y-coord";
  if (f[4] == 1) o += ",x-vel";
  if (f[5] == 1) o += ",y-vel";
  for (int k = 0; k < 4; k++)
    if (f[k] == 1) (o += ',') += sname[k];
  if (f[6] == 1) o += ",strain";
  if (f[9] == 1) o += ",disp";
  if (f[7] == 1) o += ",density";
  if (f[8] == 1) o += ",sml";
  o += "  \n";  // write(u,*) ' '
  auto col = [&](double v) {
    o += ',';
    put_f16_8(o, v);
  };
  for (int i = 0; i < nn; i++) {
    put_f16_8(o, x[2 * (size_t)i]);
    col(x[2 * (size_t)i + 1]);
    for (int k = 0; k < 2; k++)
      if (f[4 + k] == 1) col(vel[2 * (size_t)i + k]);
    for (int k = 0; k < 4; k++)
      if (f[k] == 1) col(stress[4 * (size_t)i + k]);
    if (f[6] == 1) col(iv(i));
    if (f[9] == 1) col(std::sqrt(dsp(i, 0) * dsp(i, 0) + dsp(i, 1) * dsp(i, 1)));
    if (f[7] == 1) col(rho ? rho[i] : 0.0);
    if (f[8] == 1) col(hsml ? hsml[i] : 0.0);
    o += "  \n";
  }
  if (!write_file(d + "nodes.csv." + suffix, o, false)) return SPS_ERR_ARG;
  // stress_points.csv: a comma after every column, no displacement column
  o = "x-coord,y-coord,";
  if (f[4] == 1) o += "x-vel,";
  if (f[5] == 1) o += "y-vel,";
  for (int k = 0; k < 4; k++)
    if (f[k] == 1) (o += sname[k]) += ',';
  if (f[6] == 1) o += "strain,";
  if (f[7] == 1) o += "density,";
  if (f[8] == 1) o += "sml,";
  o += "  \n";
  auto colt = [&](double v) {
    put_f16_8(o, v);
    o += ',';
  };
  for (int i = nn; i < nt; i++) {
    colt(x[2 * (size_t)i]);
    colt(x[2 * (size_t)i + 1]);
    for (int k = 0; k < 2; k++)
      if (f[4 + k] == 1) colt(vel[2 * (size_t)i + k]);
    for (int k = 0; k < 4; k++)
      if (f[k] == 1) colt(stress[4 * (size_t)i + k]);
    if (f[6] == 1) colt(iv(i));
    if (f[7] == 1) colt(rho ? rho[i] : 0.0);
    if (f[8] == 1) colt(hsml ? hsml[i] : 0.0);
    o += "  \n";
  }
  if (!write_file(d + "stress_points.csv." + suffix, o, false)) return SPS_ERR_ARG;
  // surface_points.csv: nodes with bc_or_not == 2 (list-directed lines)
  o = " x-coord,y-coord,\n";
  for (int i = 0; i < nn; i++)
    if (bc_or_not && bc_or_not[i] == 2) {
      put_ld_real(o, x[2 * (size_t)i]);
      o += " ,";
      put_ld_real(o, x[2 * (size_t)i + 1]);
      o += '\n';
    }
  if (!write_file(d + "surface_points.csv." + suffix, o, false)) return SPS_ERR_ARG;
  // GiD results: displacement (x - x00 when positions are updated, else displ) and velocity
  // always, then sxx, syy, sxy and the plastic strain as the flags select
  o.clear();
  if (!p->gid_started) {  // written by OutputMesh before the first results
    o += " GiD Post Results File 1.0\n GaussPoints \"Group1\" ElemType  Quadrilateral\n"
         " Number Of Gauss Points: 1\n Natural Coordinates: Internal\n End GaussPoints\n";
    p->gid_started = true;
  }
  auto header = [&](const char* what) {
    (o += " Result ") += what;
    put_ld_real(o, time_sph);
    o += "  Vector OnNodes \"where\" \n  Values \n";
  };
  header("\"disp\" \"disp\" ");
  for (int i = 0; i < nn; i++) {
    double dx_ = p->p.update_x ? x[2 * (size_t)i] - p->x00[2 * (size_t)i] : dsp(i, 0);
    double dy_ = p->p.update_x ? x[2 * (size_t)i + 1] - p->x00[2 * (size_t)i + 1] : dsp(i, 1);
    put_ld_int(o, i + 1);
    put_ld_real(o, dx_);
    put_ld_real(o, dy_);
    o += " 0.\n";
  }
  o += "  End Values \n";
  header("\"vel\" \"veloc\" ");
  for (int i = 0; i < nn; i++) {
    double ux = vel[2 * (size_t)i], uy = vel[2 * (size_t)i + 1];
    put_ld_int(o, i + 1);
    put_ld_real(o, ux);
    put_ld_real(o, uy);
    put_ld_real(o, std::sqrt(ux * ux + uy * uy));
    o += '\n';
  }
  o += "  End Values \n";
  const char* gname[3] = {"\"sigmaxx\" \"sxx\" ", "\"sigmayy\" \"syy\" ",
                          "\"sigmaxy\" \"sxy\" "};
  for (int k = 0; k < 3; k++)
    if (f[k] == 1) {
      header(gname[k]);
      for (int i = 0; i < nn; i++) {
        put_ld_int(o, i + 1);
        put_ld_real(o, stress[4 * (size_t)i + k]);
        o += "  0.   0.   \n";
      }
      o += "  End Values \n";
    }
  if (f[6] == 1) {
    header("\"plastic strain\" \"esp\" ");
    for (int i = 0; i < nn; i++) {
      put_ld_int(o, i + 1);
      put_ld_real(o, iv(i));
      o += "  0.  0.   \n";
    }
    o += "  End Values \n";
  }
  if (!write_file(d + p->name + ".post.res", o, true)) return SPS_ERR_ARG;
  return SPS_OK;
}

int sph_write_mesh(sph_problem* p, const char* dir) {
  if (!p || !dir) return SPS_ERR_ARG;
  const int nn = p->p.nnode;
  std::string o = " MESH    dimension 3 ElemType Quadrilateral  Nnode 4 \n  coordinates\n";
  for (int i = 0; i < nn; i++) {
    put_ld_int(o, i + 1);
    put_ld_real(o, p->x[2 * (size_t)i]);
    put_ld_real(o, p->x[2 * (size_t)i + 1]);
    put_ld_real(o, 0.0);
    o += '\n';
  }
  o += "  End coordinates\n  Elements\n";
  // the lattice cells, numbered and ordered as Read_2DMesh numbers them
  const int nx = p->ndivx, ny = p->ndivy;
  long e = 1;
  for (int i = 2; i <= nx; i++)
    for (int k = (i - 1) * ny + 2; k <= i * ny; k++) {
      put_ld_int(o, e++);
      for (long v : {(long)k, (long)k - ny, (long)k - ny - 1, (long)k - 1}) put_ld_int(o, v);
      o += "  1\n";
    }
  o += "  End elements\n";
  const std::string d = std::string(dir) + "/";
  if (!write_file(d + p->name + ".post.msh", o, false)) return SPS_ERR_ARG;
  // OutputMesh then starts the results file
  o = " GiD Post Results File 1.0\n GaussPoints \"Group1\" ElemType  Quadrilateral\n"
      " Number Of Gauss Points: 1\n Natural Coordinates: Internal\n End GaussPoints\n";
  if (!write_file(d + p->name + ".post.res", o, false)) return SPS_ERR_ARG;
  p->gid_started = true;
  return SPS_OK;
}

int sph_problem_get_arrays(sph_problem* p, sph_problem_arrays* o) {
  if (!p || !o) return SPS_ERR_ARG;
  o->ntotal2 = p->ntotal2;
  o->x = p->x.data();
  o->vel = p->vel.data();
  o->stress = p->stress.data();
  o->mass = p->mass.data();
  o->rho = p->rho.data();
  o->hsml = p->hsml.data();
  o->intvars1 = p->intvars1.data();
  o->f_drucker = p->f_drucker.data();
  o->x00 = p->x00.data();
  o->itype = p->itype.data();
  o->bc_or_not = p->bc_or_not.data();
  o->bc_info = p->bc_info.data();
  o->wall_position = p->wall_position.data();
  o->horizontal_or_not = p->horizontal_or_not.data();
  return SPS_OK;
}

int32_t sph_problem_nblocks(const sph_problem* p) { return p ? (int32_t)p->blocks.size() : 0; }

int sph_problem_block(const sph_problem* p, int32_t i, sph_run_block* out) {
  if (!p || !out || i < 0 || i >= (int32_t)p->blocks.size()) return SPS_ERR_ARG;
  *out = p->blocks[i];
  return SPS_OK;
}

const char* sph_problem_name(const sph_problem* p) { return p ? p->name.c_str() : ""; }

void sph_problem_free(sph_problem* p) { delete p; }

}  // extern "C"
