// Host object model: geometry, topology and file I/O of the MD objects, and
// the Simulation driver over the GPU engine.  Citations are to the reference
// project's files.
#include "objects.hpp"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <stdexcept>

namespace cilia {

namespace {

constexpr double kPi = 3.14159265358979323846;  // src/libcilia/abbrev.cpp:9
constexpr double kBond = 0.5;                   // Cilia::bondlength (src/cilia.h:75)

double sqdist(const double* a, const double* b) {
  double d = 0.0;
  for (int i = 0; i < 3; ++i) {
    double t = a[i] - b[i];
    d += t * t;
  }
  return d;
}

void check(int rc, mpcd_engine* e, const char* what) {
  if (rc != MPCD_OK) {
    std::string m = std::string(what) + ": " + (e ? mpcd_last_error(e) : "error");
    throw std::runtime_error(m);
  }
}

// "#name value" header of the reference's .dat files (src/libcilia/global.h:31-38)
bool read_tag(std::istream& in, const char* tag, double& v) {
  std::string garb;
  in >> garb;
  if (garb.size() < 2 || garb.substr(1) != tag) return false;
  in >> v;
  return (bool)in;
}

void write_rows(std::ostream& out, const double* a, int rows, int cols, const double* extra_col) {
  for (int r = 0; r < rows; ++r) {
    for (int c = 0; c < cols; ++c) out << a[r * cols + c] << (c + 1 < cols || extra_col ? " " : "");
    if (extra_col) out << *extra_col;
    out << "\n";
  }
}

}  // namespace

// ------------------------------------------------------------- MDObject ---

void MDObject::writedata(double globalt) {
  // MDObject::writedata (src/libcilia/mdobject.cpp:83-107)
  if (!write_data) return;
  std::ofstream data(name + ".xyz", std::ios::out | std::ios::app);
  data << (long)rodlength * num_rods << "\n";
  data << "rods: " << globalt << "\n";
  for (int i = 0; i < num_rods; ++i)
    for (int j = 0; j < rodlength; ++j) {
      const double* p = P(i, j);
      data << "C " << p[0] << " " << p[1] << " " << p[2] << "\n";
    }
}

// MDObject::save (src/libcilia/mdobject.cpp:123-139): rods x beads x 3
// positions, then velocities with the collision mass as fourth column.
void MDObject::save(std::ostream& out) const {
  out << std::setprecision(17);
  out << "#numberofrods " << num_rods << "\n#rodlength " << rodlength << "\n";
  for (int r = 0; r < num_rods; ++r) {
    write_rows(out, &pos[3 * (size_t)r * rodlength], rodlength, 3, nullptr);
    out << "\n";
  }
  out << "#velocities\n";
  for (int r = 0; r < num_rods; ++r) {
    for (int j = 0; j < rodlength; ++j) {
      const double* v = &vel[3 * ((size_t)r * rodlength + j)];
      out << v[0] << " " << v[1] << " " << v[2] << " " << (j >= startidx ? 5.0 : 0.0) << "\n";
    }
    out << "\n";
  }
}

void MDObject::save() const {
  std::ofstream out(name + ".dat");
  save(out);
}

bool MDObject::load(std::istream& in) {
  double rods = 0, len = 0;
  if (!read_tag(in, "numberofrods", rods) || !read_tag(in, "rodlength", len)) return false;
  if ((int)rods != num_rods || (int)len != rodlength) return false;
  for (size_t i = 0; i < pos.size(); ++i) in >> pos[i];
  std::string garb;
  in >> garb;
  for (long b = 0; b < nbeads(); ++b) {
    double m;
    in >> vel[3 * b] >> vel[3 * b + 1] >> vel[3 * b + 2] >> m;
  }
  return (bool)in;
}

thread_local bool MDObject::read_files = true;

bool MDObject::open_datfile() {
  if (!read_files) return false;
  std::ifstream in(name + ".dat");
  if (!in.good()) return false;
  if (!load(in)) throw std::runtime_error("cannot read " + name + ".dat");
  loaded = true;
  return true;
}

// --------------------------------------------------------------- Sphere ---

Sphere::Sphere(const libconfig::Setting& cfg)
    : Sphere((double)cfg["radius"], (double)cfg["springconstant"], (double)cfg["position"][0],
             (double)cfg["position"][1], (double)cfg["position"][2], (int)cfg["npart"],
             (std::string)cfg["name"]) {}

Sphere::Sphere(double radius, double springconstant, double wx, double wy, double wz, int npart, std::string name,
               bool write)
    : MDObject(std::move(name), 1, npart, 0, write), springconstant(springconstant), radius(radius), npart(npart) {
  int fill = 0;
  if (npart == 163) {
    fill = 2;
  } else if (npart == 643) {
    fill = 3;
  } else {
    throw std::invalid_argument("Wrong nparts has to 163 or 643");  // src/sphere.cpp:17-26
  }
  neilist.assign(npart, std::array<int, 7>{0, 0, 0, 0, 0, 0, 0});
  if (!open_datfile()) create(wx, wy, wz, fill);
}

// Sphere::create_neillist (src/sphere.cpp:264-285)
void Sphere::create_neillist(int max_part) {
  const double rcutsq = 1.1 * 1.1;
  for (int j = 0; j < max_part + 1; ++j) neilist[j].fill(0);
  for (int j = 1; j < max_part; ++j)
    for (int k = j + 1; k < max_part + 1; ++k)
      if (sqdist(P(0, j), P(0, k)) < rcutsq) {
        neilist[j][0] += 1;
        neilist[k][0] += 1;
        neilist[j][neilist[j][0]] = k;
        neilist[k][neilist[k][0]] = j;
      }
}

// Sphere::create (src/sphere.cpp:136-262): icosahedron (vertex table of the
// reference, scaled by 0.8513) refined `fill` times by edge midpoints,
// turned 90 degrees about y, projected on the sphere of `radius`.
void Sphere::create(double wx, double wy, double wz, int fill) {
  const double c5 = std::cos(2.0 * kPi / 5), s5 = std::sin(2.0 * kPi / 5);
  const double c45 = std::cos(kPi - 2.0 * 2.0 * kPi / 5), s45 = std::sin(kPi - 2.0 * 2.0 * kPi / 5);
  const double ico[12][3] = {{0., 0., 1.13},   {c5, s5, 0.50230},    {-c45, s45, 0.50230}, {-c45, -s45, 0.5023},
                             {c5, -s5, 0.50230}, {1.0, 0.0, 0.5023},   {c45, s45, -0.5023},  {-c5, s5, -0.5023},
                             {-1.0, 0.0, -0.5023}, {-c5, -s5, -0.5023}, {c45, -s45, -0.5023}, {0., 0., -1.13}};
  std::fill(pos.begin(), pos.end(), 0.0);
  std::fill(vel.begin(), vel.end(), 0.0);
  for (int i = 1; i < 13; ++i)
    for (int q = 0; q < 3; ++q) P(0, i)[q] = ico[i - 1][q] * 0.8513;
  int np = 12, tel = 12;
  for (int it = 0; it < fill; ++it) {
    create_neillist(np);
    for (int j = 1; j < np; ++j)
      for (int k = j + 1; k < np + 1; ++k)
        for (int l = 1; l < neilist[j][0] + 1; ++l)
          if (neilist[j][l] == k) {
            tel += 1;
            for (int q = 0; q < 3; ++q) P(0, tel)[q] = (P(0, j)[q] + P(0, k)[q]) / 2.0;
          }
    np = tel;
    for (int i = 1; i < np + 1; ++i)
      for (int q = 0; q < 3; ++q) P(0, i)[q] *= 2.0;
  }
  create_neillist(np);
  np++;
  for (int i = 1; i < np; ++i) {
    double* p = P(0, i);
    const double xi = p[0], zi = p[2];
    p[0] = zi;
    p[2] = -xi;
  }
  for (int i = 1; i < np; ++i) {
    double* p = P(0, i);
    const double scale = radius / std::sqrt(sqdist(p, P(0, 0)));
    for (int q = 0; q < 3; ++q) p[q] *= scale;
    p[0] = p[0] + wx;
    p[1] += wy;
    p[2] = p[2] + wz;
  }
  P(0, 0)[0] += wx;
  P(0, 0)[1] += wy;
  P(0, 0)[2] += wz;
  double hb = 0.0, norm = 0.0;
  for (int i = 1; i < np; ++i)
    for (int j = 1; j < neilist[i][0] + 1; ++j) {
      hb += std::sqrt(sqdist(P(0, i), P(0, neilist[i][j])));
      norm++;
    }
  headbond = hb / norm;
}

// Sphere::recalcforce (src/sphere.cpp:87-119): radial springs centre <-> i
// (0.1 k, rest = radius), then the mesh edges (k, rest = mean edge length)
void Sphere::emit_forces(SpringList& s) const {
  for (int i = 1; i < npart; i++) {
    s.add(bead(0, 0), bead(0, i), MPCD_SPRING_CONST, 0, radius, 0.1 * springconstant);
    s.add(bead(0, i), bead(0, 0), MPCD_SPRING_CONST, 0, radius, 0.1 * springconstant);
  }
  for (int i = 1; i < npart; i++)
    for (int j = 1; j < neilist[i][0] + 1; j++)
      s.add(bead(0, i), bead(0, neilist[i][j]), MPCD_SPRING_CONST, 0, headbond, springconstant);
}

void Sphere::save(std::ostream& out) const {
  MDObject::save(out);
  out << "#neilist\n";
  for (int i = 0; i < npart; i++) {
    for (int j = 0; j < 7; j++) out << neilist[i][j] << " ";
    out << "\n";
  }
  out << "#headbond\n" << headbond << "\n";
}

bool Sphere::load(std::istream& in) {
  if (!MDObject::load(in)) return false;
  std::string garb;
  in >> garb;
  if (garb != "#neilist") return false;
  for (int i = 0; i < rodlength; i++)
    for (int j = 0; j < 7; j++) in >> neilist[i][j];
  in >> garb;
  if (garb != "#headbond") return false;
  in >> headbond;
  return (bool)in;
}

// ---------------------------------------------------------------- Cilia ---

Cilia::Cilia(const libconfig::Setting& cfg)
    : MDObject((std::string)cfg["name"], 3, (int)cfg["rodlength"], 0, (bool)cfg["write_data"]) {
  init(cfg, (double)cfg["position"][0], (double)cfg["position"][1], (double)cfg["position"][2],
       (double)cfg["thetaX"], (double)cfg["thetaY"], (double)cfg["thetaZ"]);
}

Cilia::Cilia(const libconfig::Setting& cfg, const double* p, double tx, double ty, double tz, std::string nm,
             int sidx, int nank)
    : MDObject(std::move(nm), 3, (int)cfg["rodlength"], sidx, true) {
  num_anker = nank;
  init(cfg, p[0], p[1], p[2], tx, ty, tz);
}

// Cilia::Cilia (src/cilia.cpp:11-39)
void Cilia::init(const libconfig::Setting& cfg, double wx, double wy, double wz, double tx, double ty, double tz) {
  if (rodlength < 2) throw std::invalid_argument("rodlength must be at least 2");
  beatstrength = (double)cfg["beatstrength"];
  bending = (double)cfg["bending"];
  min_bend = (double)cfg["min_bend"];
  max_bend = (double)cfg["max_bend"];
  m_speed = (double)cfg["m_speed"];
  springconstant = (double)cfg["springconstant"];
  if (num_anker == 0) num_anker = 2;
  start = num_anker;
  midpnt = start;
  oldlength.assign(rodlength, kBond);
  if (!open_datfile()) create(wx, wy, wz, tx, ty, tz);
  newlength.assign(rodlength, kBond);
}

// Cilia::create (src/cilia.cpp:275-325)
void Cilia::create(double wx, double wy, double wz, double thetaX, double thetaY, double thetaZ) {
  std::fill(pos.begin(), pos.end(), 0.0);
  std::fill(vel.begin(), vel.end(), 0.0);
  const double l0 = kBond * std::sin(kPi / 3.0) * 2. / 3.;
  for (int i = 0; i < rodlength; ++i) {
    double* p0 = P(0, i);
    double* p1 = P(1, i);
    double* p2 = P(2, i);
    p0[2] = kBond * i;
    p0[0] -= l0;
    p1[2] = kBond * i;
    p1[1] = kBond / 2.0;
    p1[0] = kBond * std::sin(kPi / 3.0) - l0;
    p2[2] = kBond * i;
    p2[1] = -kBond / 2.0;
    p2[0] = kBond * std::sin(kPi / 3.0) - l0;
  }
  for (int j = 0; j < num_rods; ++j)
    for (int i = 0; i < rodlength; ++i) {
      double* p = P(j, i);
      const double xi = p[0], yi = p[1], zi = p[2];
      p[0] = zi * std::sin(thetaY) + std::cos(thetaY) * (xi * std::cos(thetaZ) - yi * std::sin(thetaZ));
      p[1] = std::cos(thetaX) * (yi * std::cos(thetaZ) + xi * std::sin(thetaZ)) -
             std::sin(thetaX) * (zi * std::cos(thetaY) + std::sin(thetaY) * (-(xi * std::cos(thetaZ)) + yi * std::sin(thetaZ)));
      p[2] = std::sin(thetaX) * (yi * std::cos(thetaZ) + xi * std::sin(thetaZ)) +
             std::cos(thetaX) * (zi * std::cos(thetaY) + std::sin(thetaY) * (-(xi * std::cos(thetaZ)) + yi * std::sin(thetaZ)));
    }
  for (int i = 0; i < num_rods; ++i)
    for (int j = 0; j < rodlength; ++j) {
      double* p = P(i, j);
      p[0] += wx;
      p[1] += wy;
      p[2] += wz;
    }
}

// Cilia::recalcforce + addcross (src/cilia.cpp:127-239) as spring entries.
// Bond rests of filament 0 and the diagonal rests follow the active bond
// table (refreshed on the device every 0.01 time units).
void Cilia::emit_forces(SpringList& s) const {
  const int R = rodlength;
  const double k = springconstant, cross = std::sqrt(2.0) * kBond;
  const int base = bond_base_;
  auto B = [&](int q) { return bead_offset + q; };
  for (int i = 0; i < R - 1; i++) {
    s.add(B(i), B(i + 1), MPCD_SPRING_BOND, base + i, 0.0, k);
    s.add(B(i + 1), B(i), MPCD_SPRING_BOND, base + i, 0.0, k);
    s.add(B(R + i), B(R + i + 1), MPCD_SPRING_CONST, 0, kBond, k);
    s.add(B(R + i + 1), B(R + i), MPCD_SPRING_CONST, 0, kBond, k);
    s.add(B(2 * R + i), B(2 * R + i + 1), MPCD_SPRING_CONST, 0, kBond, k);
    s.add(B(2 * R + i + 1), B(2 * R + i), MPCD_SPRING_CONST, 0, kBond, k);
  }
  for (int i = 0; i < R; ++i) {
    s.add(B(i), B(i + R), MPCD_SPRING_CONST, 0, kBond, k);
    s.add(B(i), B(i + 2 * R), MPCD_SPRING_CONST, 0, kBond, k);
    s.add(B(i + R), B(i), MPCD_SPRING_CONST, 0, kBond, k);
    s.add(B(i + R), B(i + 2 * R), MPCD_SPRING_CONST, 0, kBond, k);
    s.add(B(i + 2 * R), B(i), MPCD_SPRING_CONST, 0, kBond, k);
    s.add(B(i + 2 * R), B(i + R), MPCD_SPRING_CONST, 0, kBond, k);
  }
  for (int i = 0; i < R - 1; ++i) {
    s.add(B(i), B(i + R + 1), MPCD_SPRING_DIAG, base + i, 0.0, k);
    s.add(B(i), B(i + 2 * R + 1), MPCD_SPRING_DIAG, base + i, 0.0, k);
    s.add(B(i + R), B(i + 1), MPCD_SPRING_DIAG, base + i, 0.0, k);
    s.add(B(i + 2 * R), B(i + 1), MPCD_SPRING_DIAG, base + i, 0.0, k);
    s.add(B(i + R), B(i + 2 * R + 1), MPCD_SPRING_CONST, 0, cross, k);
    s.add(B(i + 2 * R), B(i + R + 1), MPCD_SPRING_CONST, 0, cross, k);
  }
  for (int i = 1; i < R; ++i) {
    s.add(B(i), B(i + R - 1), MPCD_SPRING_DIAG, base + i - 1, 0.0, k);
    s.add(B(i), B(i + 2 * R - 1), MPCD_SPRING_DIAG, base + i - 1, 0.0, k);
    s.add(B(i + R), B(i - 1), MPCD_SPRING_DIAG, base + i - 1, 0.0, k);
    s.add(B(i + 2 * R), B(i - 1), MPCD_SPRING_DIAG, base + i - 1, 0.0, k);
    s.add(B(i + R), B(i + 2 * R - 1), MPCD_SPRING_CONST, 0, cross, k);
    s.add(B(i + 2 * R), B(i + R - 1), MPCD_SPRING_CONST, 0, cross, k);
  }
}

void Cilia::emit_cilia(std::vector<mpcd_cilium>& c, std::vector<double>& nl, std::vector<double>& ol) const {
  mpcd_cilium d{};
  d.kind = beat_kind();
  d.rodlength = rodlength;
  d.num_anker = num_anker;
  d.bead0 = (int)bead_offset;
  d.bond_base = bond_base_;
  d.beatstrength = beatstrength;
  d.bending = bending;
  d.max_bend = max_bend;
  d.m_speed = m_speed;
  d.power_stroke_duration = power_dur();
  d.recovery_stroke_duration = recovery_dur();
  d.start = start;
  d.midpnt = midpnt;
  d.tstroke = Tstroke;
  c.push_back(d);
  nl.insert(nl.end(), newlength.begin(), newlength.end());
  ol.insert(ol.end(), oldlength.begin(), oldlength.end());
}

void Cilia::take_cilia_state(const double* st2, const double* nl, const double* ol) {
  midpnt = st2[0];
  Tstroke = st2[1];
  for (int i = 0; i < rodlength; ++i) {
    newlength[i] = nl[bond_base_ + i];
    oldlength[i] = ol[bond_base_ + i];
  }
}

void Cilia::save(std::ostream& out) const {
  MDObject::save(out);
  out << "#oldlength\n";
  for (int i = 0; i < rodlength; ++i) out << oldlength[i] << (i + 1 < rodlength ? " " : "\n");
  out << "#midpnt\n" << midpnt << "\n#tstroke\n" << Tstroke;
}

bool Cilia::load(std::istream& in) {
  if (!MDObject::load(in)) return false;
  std::string garb;
  in >> garb;
  oldlength.assign(rodlength, kBond);
  for (int i = 0; i < rodlength; ++i) in >> oldlength[i];
  in >> garb >> midpnt >> garb >> Tstroke;
  return (bool)in;
}

// ConstantBeatCilia (src/ConstantBeatCilia.h:14-21)
ConstantBeatCilia::ConstantBeatCilia(const libconfig::Setting& cfg)
    : Cilia(cfg), power_stroke_duration((double)cfg["power_stroke_duration"]),
      recovery_stroke_duration((double)cfg["recovery_stroke_duration"]) {
  if (!loaded) Tstroke = (double)cfg["start_delay"];
}

ConstantBeatCilia::ConstantBeatCilia(const libconfig::Setting& cfg, const double* p, double tx, double ty, double tz,
                                     std::string nm, int sidx, int nank)
    : Cilia(cfg, p, tx, ty, tz, std::move(nm), sidx, nank),
      power_stroke_duration((double)cfg["power_stroke_duration"]),
      recovery_stroke_duration((double)cfg["recovery_stroke_duration"]) {
  if (!loaded) Tstroke = (double)cfg["start_delay"];
}

// ---------------------------------------------------------------- Clami ---

// Clami::Clami + create_cilia (src/clami.cpp:32-150)
Clami::Clami(const libconfig::Setting& cfg, Simulation& sim) : MDObject((std::string)cfg["name"], 0, 0, 0, true) {
  double radius = 0.0;
  cfg.lookupValue("radius", radius);
  if (radius <= 0.0) throw std::invalid_argument("received negative value");
  {
    std::ifstream probe(name + ".dat");
    loaded = sim.opt.read_files && probe.good();
  }
  double p[3] = {(double)cfg["position"][0], (double)cfg["position"][1], (double)cfg["position"][2]};
  cfg.lookupValue("springconstant", springconstant);
  cfg["springconstant"] = 20000.0;  // the reference writes this back into the cfg (clami.cpp:50)
  sphere = new Sphere(radius, springconstant, p[0], p[1], p[2], 643, name + "_sphere", false);
  sim.add_md_object(sphere);
  const int nxl = cfg["num_equators"].getLength();
  const int nyl = cfg["y_thetas"].getLength();
  const int noff = cfg["theta_offset"].getLength();
  if (nxl != nyl || nxl != noff) throw std::runtime_error("config error: Num of offsets mismatch");
  int num_cilia = 0;
  for (int i = 0; i < nyl; i++) num_cilia += (int)cfg["num_equators"][i];
  const bool delays = cfg.exists("start_delays");
  if (delays && num_cilia != cfg["start_delays"].getLength())
    throw std::runtime_error("config error: start_delays length differs from the number of cilia");
  const libconfig::Setting& ccfg = cfg["cilia"];
  int cil_idx = 0;
  for (int i = 0; i < nyl; i++) {
    double thetaY = (double)cfg["y_thetas"][i];
    thetaY *= kPi / 180.;
    const double off = (double)cfg["theta_offset"][i];
    const int nx = (int)cfg["num_equators"][i];
    for (int j = 0; j < nx; j++) {
      const double thetaX = off + 2 * kPi * j / nx;
      const double start_delay = delays ? (double)cfg["start_delays"][cil_idx] : 0.0;
      const int wo = 3;
      const double r = sphere->radius - wo * kBond;
      double pc[3] = {r * std::sin(thetaY), -r * std::cos(thetaY) * std::sin(thetaX), r * std::cos(thetaX) * std::cos(thetaY)};
      for (int q = 0; q < 3; ++q) pc[q] += p[q];
      const libconfig::Setting& cc = ccfg;
      cc["name"] = name + "_cilia" + std::to_string(cil_idx);
      cc["position"][0] = pc[0];
      cc["position"][1] = pc[1];
      cc["position"][2] = pc[2];
      cc["thetaX"] = thetaX;
      cc["thetaY"] = thetaY;
      cc["thetaZ"] = (double)ccfg["thetaZ"];
      cc["start_delay"] = start_delay;
      MDObject* obj = sim.add_md_object(cc);
      Cilia* c = dynamic_cast<Cilia*>(obj);
      if (c == nullptr) throw std::runtime_error("config error: Clami cilia must be Cilia or ConstantBeatCilia");
      if (!loaded) {
        const int wod = (int)(wo * kBond / kBond);
        attach(c, (int)cilias.size(), 0);
        attach(c, (int)cilias.size(), wod);
      }
      cilias.push_back(c);
      cil_idx++;
    }
  }
  num_particles = sphere->nbeads();
  for (Cilia* c : cilias) num_particles += c->nbeads();
  if (loaded) {
    std::ifstream in(name + ".dat");
    if (!load(in)) throw std::runtime_error("cannot read " + name + ".dat");
  }
}

// Clami::add_springs_for_rods_idx (src/clami.cpp:152-174): the nearest sphere
// bead (Matrix::get_closest_idx, Matrix.h:602-615) and its neighbours
// 1..count-1; rest lengths are the initial distances.
void Clami::attach(Cilia* c, int cidx, int wo) {
  for (int j = 0; j < c->num_rods; ++j) {
    const double* pc = c->P(j, wo);
    double min_dist = 9999;
    int idx = 0;
    for (int i = 0; i < sphere->rodlength; ++i) {
      const double d = sqdist(sphere->P(0, i), pc);
      if (min_dist > d) {
        min_dist = d;
        idx = i;
      }
    }
    springs.push_back(Attach{cidx, idx, j, wo, std::sqrt(sqdist(sphere->P(0, idx), pc))});
    for (int n = 1; n < sphere->neilist[idx][0]; ++n) {
      const int sb = sphere->neilist[idx][n];
      springs.push_back(Attach{cidx, sb, j, wo, std::sqrt(sqdist(sphere->P(0, sb), pc))});
    }
  }
}

// Clami::global_forces (src/clami.cpp:188-198): F = spring(sphere, cilium)
// added to the sphere bead and subtracted from the cilium bead; both halves
// are one-sided entries with the zero-distance guard of the vector spring.
void Clami::emit_global_forces(SpringList& s) const {
  for (const Attach& a : springs) {
    const long sb = sphere->bead(0, a.sphere_bead);
    const long cb = cilias[a.cil]->bead(a.rod, a.bead);
    s.add(sb, cb, MPCD_SPRING_GUARDED, 0, a.l0, springconstant);
    s.add(cb, sb, MPCD_SPRING_GUARDED, 0, a.l0, springconstant);
  }
}

// Clami::writedata (src/clami.cpp:208-284): .xyz frame of the cilia and one
// .san line: time, centre of mass, its velocity, body frame n, b, p from
// sphere beads 1, 32, 137 relative to bead 0, dissipated power.
void Clami::writedata(double globalt) {
  std::ofstream data(name + ".xyz", std::ios::out | std::ios::app);
  double xcm[3] = {0, 0, 0}, vcm[3] = {0, 0, 0};
  const int even = cilias.empty() ? 0 : cilias[0]->rodlength % 2;
  if (!cilias.empty())
    data << cilias.size() * cilias[0]->num_rods * (cilias[0]->rodlength / 2 + even) << "\n";
  else
    data << 0 << "\n";
  data << "rods: " << globalt << "\n";
  for (long b = 0; b < sphere->nbeads(); ++b)
    for (int q = 0; q < 3; ++q) {
      xcm[q] += sphere->pos[3 * b + q];
      vcm[q] += sphere->vel[3 * b + q];
    }
  for (Cilia* c : cilias) {
    for (int i = 0; i < c->num_rods; ++i)
      for (int j = 0; j < c->rodlength; ++j) {
        const double* p = c->P(i, j);
        if ((j + 1) % 2 == even) data << (i == 0 ? "H " : "O ") << p[0] << " " << p[1] << " " << p[2] << "\n";
        for (int q = 0; q < 3; ++q) {
          xcm[q] += p[q];
          vcm[q] += c->vel[3 * ((size_t)i * c->rodlength + j) + q];
        }
      }
  }
  data.close();
  for (int q = 0; q < 3; ++q) {
    xcm[q] /= num_particles;
    vcm[q] /= num_particles;
  }
  const double* s0 = sphere->P(0, 0);
  double n[3], bb[3], pp[3];
  for (int q = 0; q < 3; ++q) {
    n[q] = sphere->P(0, 1)[q] - s0[q];
    bb[q] = sphere->P(0, 32)[q] - s0[q];
    pp[q] = sphere->P(0, 137)[q] - s0[q];
  }
  std::ofstream san(name + ".san", std::ios::out | std::ios::app);
  san << globalt << " " << xcm[0] << " " << xcm[1] << " " << xcm[2] << " " << vcm[0] << " " << vcm[1] << " "
      << vcm[2] << " " << n[0] << " " << n[1] << " " << n[2] << " " << bb[0] << " " << bb[1] << " " << bb[2] << " "
      << pp[0] << " " << pp[1] << " " << pp[2] << " " << diss_energy_interval / measureinterval / tstep << "\n";
}

// Clami::save / load (src/clami.cpp:288-345): attachment springs only
void Clami::save(std::ostream& out) const {
  out << std::setprecision(17) << "#springs\n" << cilias.size() << "\n";
  for (const Attach& a : springs)
    out << a.cil << " " << a.sphere_bead << " " << (a.rod * cilias[a.cil]->rodlength + a.bead) << " " << a.l0 << "\n";
}

bool Clami::load(std::istream& in) {
  std::string garb;
  in >> garb;
  if (garb != "#springs") return false;
  size_t nc = 0;
  in >> nc;
  if (nc != cilias.size()) return false;
  springs.clear();
  int ci, sb, cb;
  double l0;
  while (in >> ci >> sb >> cb >> l0) {
    if (ci < 0 || ci >= (int)cilias.size()) return false;
    const int len = cilias[ci]->rodlength;
    springs.push_back(Attach{ci, sb, cb / len, cb % len, l0});
  }
  return true;
}

// ---------------------------------------------------------------- World ---

void World::loadparameter(const libconfig::Setting& root) {
  // World::loadparameter (src/libcilia/global.cpp:21-30)
  globalt = (double)root["globalt"];
  desiredt = (double)root["desiredt"];
  omega = (double)root["omega"];
  sizex = (int)root["sizex"];
  sizey = (int)root["sizey"];
  sizez = (int)root["sizez"];
  runtime = (double)root["runtime"];
  tstep = (double)root["tstep"];
}

void World::saveparameter(libconfig::Setting& root) const {
  root["globalt"] = globalt;
  root["desiredt"] = desiredt;
  root["runtime"] = runtime;
  root["omega"] = omega;
  root["sizex"] = sizex;
  root["sizey"] = sizey;
  root["sizez"] = sizez;
}

void add_to_batch(mpcd_batch* b, const HostSystem& h, long nbeads, int* replica) {
  mpcd_params p = h.p;
  p.precision = MPCD_FP32;
  int r = -1;
  if (mpcd_batch_add(b, &p, &r) != MPCD_OK) throw std::runtime_error(std::string("batch: ") + mpcd_batch_last_error(b));
  auto ck = [&](int rc) {
    if (rc != MPCD_OK) {
      const std::string m = std::string("batch: ") + mpcd_batch_last_error(b);
      mpcd_batch_remove(b, r);
      throw std::runtime_error(m);
    }
  };
  ck(mpcd_batch_set_shift(b, r, h.a));
  ck(mpcd_batch_set_time(b, r, h.globalt));
  const long nf = (long)h.fpos.size() / 3;
  if (nf > 0) ck(mpcd_batch_set_fluid(b, r, nf, h.fpos.data(), h.fvel.data()));
  if (nbeads > 0) {
    const SpringList& sp = h.springs;
    ck(mpcd_batch_set_beads(b, r, nbeads, h.bpos.data(), h.bvel.data(), h.moves.data()));
    ck(mpcd_batch_set_springs(b, r, (long)sp.size(), sp.target.data(), sp.other.data(), sp.kind.data(),
                              sp.ref.data(), sp.rest.data(), sp.k.data()));
    ck(mpcd_batch_set_cilia(b, r, (int)h.cilia.size(), h.cilia.data(), h.newlen.data(), h.oldlen.data()));
  }
  *replica = r;
}

// ----------------------------------------------------------- Simulation ---

Simulation::Simulation(const libconfig::Setting& root, const SimOptions& o) : opt(o) {
  MDObject::read_files = opt.read_files != 0;
  wc.loadparameter(root);
  double ststep = 0.001;  // World::ststep (src/libcilia/global.cpp:11)
  root.lookupValue("ststep", ststep);
  if (opt.ststep > 0) ststep = opt.ststep;
  wc.ststep = ststep;
  long long cfg_seed = 0;
  if (opt.seed) {
    seed = opt.seed;
  } else if (root.lookupValue("seed", cfg_seed) && cfg_seed > 0) {
    seed = (uint64_t)cfg_seed;
  } else {
    std::random_device rd;
    seed = ((uint64_t)rd() << 32) ^ rd();
  }
  rng.reset(new HostRng((uint32_t)(seed ^ (seed >> 32))));

  mpcd_params p{};
  p.sizes[0] = wc.sizex;
  p.sizes[1] = wc.sizey;
  p.sizes[2] = wc.sizez;
  p.tstep = wc.tstep;
  p.ststep = wc.ststep;
  p.precision = opt.precision;
  p.walls = opt.walls;
  p.gravity = opt.gravity;
  p.omega = wc.omega;
  p.bead_mass = opt.bead_mass;
  p.seed = seed;
  p.device = opt.device;
  p.sort_interval = opt.sort_interval;
  p.md_split = opt.md_split;
  if (opt.host_only) {
    host.p = p;
    host.globalt = wc.globalt;
  } else {
    check(mpcd_create(&p, &eng), eng, "mpcd_create");
    mpcd_set_time(eng, wc.globalt);
  }
  // MPCD::MPCD: grid shift from mpcd.dat or three draws (src/libcilia/mpcd.cpp:86-97).
  // When the file exists the reference draws nothing and reads three values
  // with plain stream extraction; its destructor writes the address of the
  // shift array (mpcd.cpp:396-403, `out << a` of a double*), from which the
  // first extraction reads 0 and the next fails, leaving 0 and then an
  // unset value.  Here every value a failed extraction leaves is 0, so such a
  // file gives the shift (0, 0, 0); a shift outside [0, 1) is wrapped into it
  // (the same cell partition, renumbered).
  double a[3] = {0.0, 0.0, 0.0};
  bool have = false;
  if (opt.read_files) {
    std::ifstream in("mpcd.dat");
    if (in.good()) {
      have = true;
      for (double& q : a) {
        if (!(in >> q)) q = 0.0;
        if (!std::isfinite(q)) q = 0.0;
        q -= std::floor(q);
        if (q >= 1.0) q = 0.0;
      }
    }
  }
  if (!have)
    for (double& q : a) q = rng->rnd();
  if (opt.host_only)
    std::memcpy(host.a, a, sizeof host.a);
  else
    check(mpcd_set_shift(eng, a), eng, "mpcd_set_shift");
  // Simulation::load_config (src/simulation.cpp:614-648)
  const libconfig::Setting& objs = root["md_objects"];
  for (int i = 0; i < objs.getLength(); ++i) {
    const libconfig::Setting& c = objs[i];
    std::string type, name;
    if (!(c.lookupValue("type", type) && c.lookupValue("name", name))) continue;
    add_md_object(c);
  }
  // Fluid::FluidFromFile (src/libcilia/fluid.cpp:21-48)
  if (opt.create_fluid) {
    if (!(opt.read_files && load_fluid("fluid_n.dat"))) create_fluid();
  }
  upload_md();
  // contact forces between cilia: the reference's -DREPELLING=eps as a cfg key
  //   repelling = <eps>;
  double repel = 0.0;
  if (!opt.host_only && root.lookupValue("repelling", repel) && repel != 0.0)
    check(mpcd_set_repelling(eng, repel), eng, "mpcd_set_repelling");
  // rigid no-slip spheres (an addition to the reference's cfg schema):
  //   rigid_spheres = ( { position = [x, y, z]; radius = r; mass = m; velocity = [..]; omega = [..]; } );
  // mass > 0 free, absent or <= 0 held (mpcd_set_rigid_spheres)
  if (root.exists("rigid_spheres") && !opt.host_only) {
    const libconfig::Setting& rs = root["rigid_spheres"];
    std::vector<mpcd_rigid_sphere> sp(rs.getLength());
    for (int i = 0; i < rs.getLength(); ++i) {
      const libconfig::Setting& c = rs[i];
      mpcd_rigid_sphere& q = sp[i];
      q = mpcd_rigid_sphere{};
      for (int j = 0; j < 3; ++j) q.center[j] = (double)c["position"][j];
      q.radius = (double)c["radius"];
      c.lookupValue("mass", q.mass);
      if (c.exists("velocity"))
        for (int j = 0; j < 3; ++j) q.velocity[j] = (double)c["velocity"][j];
      if (c.exists("omega"))
        for (int j = 0; j < 3; ++j) q.omega[j] = (double)c["omega"][j];
    }
    check(mpcd_set_rigid_spheres(eng, (int)sp.size(), sp.data()), eng, "mpcd_set_rigid_spheres");
  }
}

Simulation::~Simulation() {
  if (eng) mpcd_destroy(eng);
}

// Simulation::add_md_object (src/simulation.cpp:652-673)
MDObject* Simulation::add_md_object(const libconfig::Setting& cfg) {
  const std::string type = (std::string)cfg["type"];
  MDObject* obj = nullptr;
  if (type == "Clami") {
    obj = new Clami(cfg, *this);
  } else if (type == "Sphere") {
    obj = new Sphere(cfg);
  } else if (type == "Cilia") {
    obj = new Cilia(cfg);
  } else if (type == "ConstantBeatCilia") {
    obj = new ConstantBeatCilia(cfg);
  } else {
    throw std::runtime_error("Syntax Error: Unkown type:" + type);
  }
  add_md_object(obj);
  return obj;
}

void Simulation::add_md_object(MDObject* obj) {
  obj->bead_offset = nbeads;
  nbeads += obj->nbeads();
  md_objects.emplace_back(obj);
}

void Simulation::upload_md() {
  std::vector<double> P, V;
  std::vector<int> moves;
  int bond_base = 0;
  for (auto& o : md_objects) {
    P.insert(P.end(), o->pos.begin(), o->pos.end());
    V.insert(V.end(), o->vel.begin(), o->vel.end());
    for (int r = 0; r < o->num_rods; ++r)
      for (int j = 0; j < o->rodlength; ++j) moves.push_back(j >= o->startidx ? 1 : 0);
    if (Cilia* c = dynamic_cast<Cilia*>(o.get())) {
      c->bond_base_ = bond_base;
      bond_base += c->rodlength;
    }
  }
  SpringList s;
  for (auto& o : md_objects) o->emit_forces(s);
  for (auto& o : md_objects) o->emit_global_forces(s);
  std::vector<mpcd_cilium> cil;
  std::vector<double> nl, ol;
  for (auto& o : md_objects) o->emit_cilia(cil, nl, ol);
  if (opt.host_only) {
    host.bpos = P;
    host.bvel = V;
    host.moves = moves;
    host.springs = s;
    host.cilia = cil;
    host.newlen = nl;
    host.oldlen = ol;
    return;
  }
  check(mpcd_set_beads(eng, nbeads, P.data(), V.data(), moves.data()), eng, "mpcd_set_beads");
  check(mpcd_set_springs(eng, (long)s.size(), s.target.data(), s.other.data(), s.kind.data(), s.ref.data(),
                         s.rest.data(), s.k.data()),
        eng, "mpcd_set_springs");
  check(mpcd_set_cilia(eng, (int)cil.size(), cil.data(), nl.data(), ol.data()), eng, "mpcd_set_cilia");
}

void Simulation::sync_from_device() {
  if (nbeads == 0) return;
  std::vector<double> P(3 * nbeads), V(3 * nbeads);
  check(mpcd_get_beads(eng, nbeads, P.data(), V.data()), eng, "mpcd_get_beads");
  for (auto& o : md_objects) {
    const long n = o->nbeads();
    std::copy(P.begin() + 3 * o->bead_offset, P.begin() + 3 * (o->bead_offset + n), o->pos.begin());
    std::copy(V.begin() + 3 * o->bead_offset, V.begin() + 3 * (o->bead_offset + n), o->vel.begin());
  }
  int nc = 0;
  for (auto& o : md_objects)
    if (dynamic_cast<Cilia*>(o.get())) nc++;
  if (nc) {
    std::vector<double> st(2 * nc);
    size_t nbond = 0;
    for (auto& o : md_objects)
      if (Cilia* c = dynamic_cast<Cilia*>(o.get())) nbond += c->rodlength;
    std::vector<double> nl(nbond), ol(nbond);
    check(mpcd_get_cilia(eng, nc, st.data(), nl.data(), ol.data()), eng, "mpcd_get_cilia");
    int k = 0;
    for (auto& o : md_objects)
      if (Cilia* c = dynamic_cast<Cilia*>(o.get())) {
        c->take_cilia_state(&st[2 * k], nl.data(), ol.data());
        k++;
      }
  }
}

int Simulation::next_tstep(const mpcd_inject* inj) {
  int rc = mpcd_step(eng, inj);
  if (rc == MPCD_OK) mpcd_get_time(eng, &wc.globalt);
  return rc;
}

// Fluid::create (src/libcilia/fluid.cpp:55-98): rho = 10 per cell, positions
// uniform, velocities Maxwell-Boltzmann at kT = 1, centre-of-mass velocity removed
void Simulation::create_fluid() {
  const long n = (long)wc.sizex * wc.sizey * wc.sizez * 10;
  std::vector<double> P(3 * n), V(3 * n);
  const int L[3] = {wc.sizex, wc.sizey, wc.sizez};
  for (long i = 0; i < n; ++i) {
    for (int q = 0; q < 3; ++q) P[3 * i + q] = rng->rnd() * L[q] * 1.0;
    for (int q = 0; q < 3; ++q) V[3 * i + q] = rng->normalrand() * std::sqrt(1.0);
  }
  double cm[3] = {0, 0, 0};
  for (long i = 0; i < n; ++i)
    for (int q = 0; q < 3; ++q) cm[q] += V[3 * i + q];
  for (int q = 0; q < 3; ++q) cm[q] /= n;
  for (long i = 0; i < n; ++i)
    for (int q = 0; q < 3; ++q) V[3 * i + q] -= cm[q];
  if (opt.host_only) {
    host.fpos.swap(P);
    host.fvel.swap(V);
    return;
  }
  check(mpcd_set_fluid(eng, n, P.data(), V.data()), eng, "mpcd_set_fluid");
}

// fluid_n.dat: "#numberofparticles N", positions, "#velocities", velocities with mass
// (src/libcilia/fluid.cpp:100-150)
bool Simulation::load_fluid(const char* path) {
  std::ifstream in(path);
  if (!in.good()) return false;
  double nd = 0;
  if (!read_tag(in, "numberofparticles", nd)) throw std::runtime_error("error with fluid file header");
  const long n = (long)nd;
  const long want = (long)wc.sizex * wc.sizey * wc.sizez * 10;
  if (n > want) throw std::runtime_error("Fluidfile to big.");
  std::vector<double> P(3 * n), V(3 * n);
  for (long i = 0; i < 3 * n; ++i) in >> P[i];
  std::string garb;
  in >> garb;
  for (long i = 0; i < n; ++i) {
    double m;
    in >> V[3 * i] >> V[3 * i + 1] >> V[3 * i + 2] >> m;
  }
  if (!in) throw std::runtime_error("cannot read fluid file");
  if (opt.host_only) {
    host.fpos.swap(P);
    host.fvel.swap(V);
    return true;
  }
  check(mpcd_set_fluid(eng, n, P.data(), V.data()), eng, "mpcd_set_fluid");
  return true;
}

void Simulation::save_fluid(const char* path) const {
  const long n = mpcd_fluid_count(eng);
  std::vector<double> P(3 * n), V(3 * n);
  check(mpcd_get_fluid(eng, n, P.data(), V.data()), eng, "mpcd_get_fluid");
  std::ofstream out(path);
  out << std::scientific << std::setprecision(17);
  out << "#numberofparticles " << n << "\n";
  for (long i = 0; i < n; ++i) out << P[3 * i] << " " << P[3 * i + 1] << " " << P[3 * i + 2] << "\n";
  out << "\n#velocities\n";
  for (long i = 0; i < n; ++i) out << V[3 * i] << " " << V[3 * i + 1] << " " << V[3 * i + 2] << " " << 1.0 << "\n";
}

// Simulation::~Simulation saves: objects, fluid, grid shift (src/simulation.cpp:354-380,
// src/libcilia/mpcd.cpp:396-403)
void Simulation::save_all() const {
  for (auto& o : md_objects) o->save();
  save_fluid("fluid_n.dat");
  double a[3];
  mpcd_get_shift(eng, a);
  std::ofstream out("mpcd.dat");
  out << std::setprecision(17) << a[0] << " " << a[1] << " " << a[2] << "\n";
}

// MPCD::debug (src/libcilia/mpcd.cpp:404-467): totals appended to mpcd.san
void Simulation::debug(const char* path) {
  mpcd_obs o{};
  check(mpcd_observables(eng, &o), eng, "mpcd_observables");
  std::cout << "Total Momentum \t= " << o.momentum[0] << " " << o.momentum[1] << " " << o.momentum[2] << "\n"
            << "Total Number \t= " << (long)o.n << "\nTotal Mass \t= " << o.mass << "\nkbT \t= " << o.kT << "\n\n";
  std::ofstream data(path, std::ios::out | std::ios::app);
  data << wc.globalt << " " << o.diss_energy << " " << (long)o.n << " " << o.mass << " " << o.momentum[0] << " "
       << o.momentum[1] << " " << o.momentum[2] << " " << o.kT << "\n";
}

// What Simulation::run writes after a measure interval (src/simulation.cpp:
// 103-107): every object's writedata (a Clami's dissipated power from the
// energy the thermostat removed since the last interval, which is then
// cleared, as Clami::writedata clears MPCD::diss_energy_total); with
// debug_row, then MPCD::debug's line in mpcd.san.
void Simulation::write_measure(bool objects, bool debug_row) {
  mpcd_obs o{};
  check(mpcd_observables(eng, &o), eng, "mpcd_observables");
  sync_from_device();
  if (objects) {
    for (auto& obj : md_objects) {
      if (Clami* c = dynamic_cast<Clami*>(obj.get())) {
        c->diss_energy_interval = o.diss_energy;
        c->tstep = wc.tstep;
        c->measureinterval = wc.measureinterval;
      }
      obj->writedata(wc.globalt);
    }
    check(mpcd_reset_diss(eng), eng, "mpcd_reset_diss");
  }
  if (debug_row) debug("mpcd.san");
}

void Simulation::write_fluid_temp(const char* path) {
  mpcd_obs o{};
  check(mpcd_observables(eng, &o), eng, "mpcd_observables");
  std::ofstream data(path, std::ios::out | std::ios::app);
  data << o.fluid_T << "\n";
}

// Simulation::run (src/simulation.cpp:59-156): measure interval of 50 MPC
// steps, writedata of every object, fps report, save every 7200 s of wall
// time, stop at desiredt or when the runtime budget is used.
void Simulation::run() {
  using clk = std::chrono::steady_clock;
  const auto started = clk::now();
  auto lastsave = started;
  const double t_begin = wc.globalt;
  std::cout << "start simulation:" << std::endl;
  while (wc.globalt < wc.desiredt) {
    const auto t0 = clk::now();
    for (int s = 0; s < wc.measureinterval; ++s) check(next_tstep(nullptr), eng, "mpcd_step");
    write_measure(true, false);
    const double ms = std::chrono::duration<double, std::milli>(clk::now() - t0).count();
    std::cout << "T =" << wc.globalt;
    if (ms > 0) std::cout << " (" << 1000.0 * wc.tstep * wc.measureinterval / ms << "fps)";
    std::cout << std::endl;
    const double since_save = std::chrono::duration<double>(clk::now() - lastsave).count();
    const double elapsed = std::chrono::duration<double>(clk::now() - started).count();
    if (since_save > 7200 || elapsed > wc.runtime) {
      if (elapsed > wc.runtime) break;
      save_all();
      lastsave = clk::now();
    }
  }
  const double elapsed = std::chrono::duration<double>(clk::now() - started).count();
  std::cout << "\n\nend simulation:\n" << wc.globalt - t_begin << " r:" << elapsed << "\n"
            << "fps: " << (elapsed > 0 ? (wc.globalt - t_begin) / elapsed : 0.0) << std::endl;
}

}  // namespace cilia
