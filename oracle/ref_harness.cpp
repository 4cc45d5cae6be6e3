// Oracle harness around the reference implementation (test infrastructure).
//
// Built by oracle/Makefile together with the reference's own translation units
// (src/simulation.cpp, src/cilia.cpp, src/sphere.cpp, src/clami.cpp,
// src/ConstantBeatCilia.cpp, src/libcilia/{fluid,mdobject,globalforces}.cpp,
// compiled unmodified with the flags of src/Makefile:2-10) into oracle/_ref/.
// This translation unit includes src/libcilia/mpcd.cpp directly (like
// src/main.cpp:24-26 includes basicf.cpp/global.cpp) so that it can call the
// reference's own `rgamma` (src/libcilia/mpcd.cpp:13-43).
//
// Modes
//   ref_harness kat <seed> <count>            MT19937 outputs of the reference MTRand
//   ref_harness gamma <seed> <Nc> <count>     rgamma(Nc) samples (src/libcilia/mpcd.cpp:13-43)
//   ref_harness run <cfg> <outdir> <seed> <nsteps> <ststep> <dump_list>
//       Builds Simulation(root) from <cfg> exactly like src/main.cpp:48-98 (one
//       OpenMP thread, randi[0] = MTRand(seed)), then runs <nsteps> MPC steps
//       through Simulation::next_tstep (src/simulation.cpp:217-265).  Before
//       each step it replays the collision's random draws on a clone of the
//       generator, in the consumption order of src/libcilia/mpcd.cpp:148-212, to
//       record the per-cell Gamma variate and rotation axis (and, in the walls
//       build, the virtual-particle momentum of wall-layer cells), and checks
//       afterwards that the real step consumed exactly those draws.  It writes
//       raw little-endian float64 arrays plus index.txt into <outdir>.
//   ref_harness run ... <dump_list> <write_list>
//       also calls every object's writedata (Clami: <name>.xyz and <name>.san,
//       src/clami.cpp:208-284) and MPCD::debug (mpcd.san, src/libcilia/mpcd.cpp:
//       404-467) after the steps of <write_list>, as Simulation::run does after
//       a measure interval (src/simulation.cpp:76-107).
#include <omp.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cassert>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "libconfig.h++"

#define private public
#define protected public
#include "abbrev.cpp"
#include "basicf.cpp"
#include "global.cpp"
#include "simulation.h"
#include "mpcd.cpp"
#include "cilia.h"
#include "sphere.h"
#include "clami.h"
#include "ConstantBeatCilia.h"
#undef private
#undef protected

namespace {

struct Out {
  std::string dir;
  std::ofstream index;
  explicit Out(const std::string& d) : dir(d), index(d + "/index.txt") {}
  void put(const std::string& name, const double* p, const std::vector<long>& shape) {
    long n = 1;
    for (long s : shape) n *= s;
    std::ofstream f(dir + "/" + name + ".f64", std::ios::binary);
    f.write(reinterpret_cast<const char*>(p), n * sizeof(double));
    index << name;
    for (long s : shape) index << " " << s;
    index << "\n";
  }
  void put(const std::string& name, const std::vector<double>& v, const std::vector<long>& shape) {
    put(name, v.data(), shape);
  }
};

bool same_state(MTRand& a, MTRand& b) {
  MTRand::uint32 sa[MTRand::SAVE], sb[MTRand::SAVE];
  a.save(sa);
  b.save(sb);
  return std::memcmp(sa, sb, sizeof sa) == 0;
}

// Replays the collision's draws (src/libcilia/mpcd.cpp:148-212) on a clone of
// randi[0].  gamma[c] = Gamma variate, -1 if the cell was not thermostatted
// (E_rel <= 0 or N_c <= 1), -2 if the cell was empty.  axis[c] = rotation axis.
void replay_collision(Simulation& sim, MTRand& clone, std::vector<double>& gamma,
                      std::vector<double>& axis, std::vector<double>& virt) {
  MPCD& m = sim.mpcd;
  MTRand* orig = randi[0];
  MTRand::uint32 st[MTRand::SAVE];
  orig->save(st);
  clone.load(st);
  randi[0] = &clone;
  const int ncell = m.numberofboxes;
  gamma.assign(ncell, -2.0);
  axis.assign(3 * (size_t)ncell, 0.0);
  virt.assign(3 * (size_t)ncell, 0.0);
  for (int cid = 0; cid < ncell; ++cid) {
    double ux = 0, uy = 0, uz = 0, le = 0;
    int num = 0, masse = 0;
    for (unsigned vid = 0; vid < m.boxes[0][cid].size(); ++vid) {
      double* v = m.boxes[0][cid][vid];
      const double pm = v[3];
      ux += v[0] * pm;
      uy += v[1] * pm;
      uz += v[2] * pm;
      masse += pm;
      le += pm * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    }
    num += m.boxes[0][cid].size();
    if (num > 0) {
#if defined(SLIP) || defined(NOSLIP)
      // wall layers: virtual particles, drawn before the Gamma variate (mpcd.cpp:175-198)
      if ((cid < m.size[0] * m.size[1]) or (cid > m.size[0] * m.size[1] * (m.size[2] - 1))) {
        if (num < MPCD::rho) {
          const int dm = MPCD::rho - num;
          for (int q = 0; q < 3; ++q) virt[3 * cid + q] = sqrt(dm * MPCD::temp) * normalrand();
          ux += virt[3 * cid + 0];
          uy += virt[3 * cid + 1];
          uz += virt[3 * cid + 2];
          masse += dm;
          num += dm;
          le += (virt[3 * cid] * virt[3 * cid] + virt[3 * cid + 1] * virt[3 * cid + 1] +
                 virt[3 * cid + 2] * virt[3 * cid + 2]) /
                dm;
        }
      }
#endif
      ux /= masse;
      uy /= masse;
      uz /= masse;
      double rel = le - (ux * ux + uy * uy + uz * uz) * masse;
      if (rel > 0 and num > 1) {
        gamma[cid] = rgamma(num);
      } else {
        gamma[cid] = -1.0;
      }
      double phi = 2 * PI * randi[0]->rand();
      double theta = 2.0 * randi[0]->rand() - 1.0;
      double s1 = sqrt(1.0 - theta * theta);
      axis[3 * cid + 0] = s1 * cos(phi);
      axis[3 * cid + 1] = s1 * sin(phi);
      axis[3 * cid + 2] = theta;
    }
  }
  randi[0] = orig;
}

void dump_state(Out& out, Simulation& sim, const std::string& tag) {
  Fluid& fl = *sim.fluid;
  const long n = fl.numberofparticles;
  std::vector<double> pos(3 * n), vel(3 * n);
  for (long i = 0; i < n; ++i)
    for (int q = 0; q < 3; ++q) {
      pos[3 * i + q] = fl.positions[i][q];
      vel[3 * i + q] = fl.velocities[i][q];
    }
  out.put(tag + "_fluid_pos", pos, {n, 3});
  out.put(tag + "_fluid_vel", vel, {n, 3});
  for (size_t k = 0; k < sim.md_objects.size(); ++k) {
    MDObject* o = sim.md_objects[k];
    const long rods = o->num_rods, len = o->rodlength;
    if (rods * len == 0) continue;
    std::vector<double> p(rods * len * 3), v(rods * len * 3);
    for (long r = 0; r < rods; ++r)
      for (long j = 0; j < len; ++j)
        for (int q = 0; q < 3; ++q) {
          p[(r * len + j) * 3 + q] = o->positions[r][j][q];
          v[(r * len + j) * 3 + q] = o->velocities[r][j][q];
        }
    out.put(tag + "_obj" + std::to_string(k) + "_pos", p, {rods, len, 3});
    out.put(tag + "_obj" + std::to_string(k) + "_vel", v, {rods, len, 3});
    Cilia* c = dynamic_cast<Cilia*>(o);
    if (c != nullptr) {
      std::vector<double> s(2 * len + 2);
      for (long j = 0; j < len; ++j) {
        s[j] = c->newlength[j];
        s[len + j] = c->oldlength[j];
      }
      s[2 * len] = c->midpnt;
      s[2 * len + 1] = c->Tstroke;
      out.put(tag + "_obj" + std::to_string(k) + "_cilstate", s, {2 * len + 2});
    }
  }
  double meta[3] = {wc.globalt, (double)sim.mpcd.diss_energy_total, 0.0};
  out.put(tag + "_meta", meta, {3});
}

int run_mode(int argc, char** argv) {
  if (argc < 8) {
    std::cerr << "usage: ref_harness run <cfg> <outdir> <seed> <nsteps> <ststep> <dump_list>\n";
    return 2;
  }
  std::string cfgpath = argv[2];
  std::string outdir = argv[3];
  unsigned long seed = std::strtoul(argv[4], nullptr, 10);
  int nsteps = std::atoi(argv[5]);
  double ststep = std::atof(argv[6]);
  std::vector<int> dumps, writes;
  {
    std::stringstream ss(argv[7]);
    std::string tok;
    while (std::getline(ss, tok, ',')) dumps.push_back(std::atoi(tok.c_str()));
  }
  if (argc > 8) {
    std::stringstream ss(argv[8]);
    std::string tok;
    while (std::getline(ss, tok, ',')) writes.push_back(std::atoi(tok.c_str()));
  }
  char absbuf[4096];
  if (realpath(cfgpath.c_str(), absbuf) == nullptr) {
    std::cerr << "cannot resolve " << cfgpath << "\n";
    return 2;
  }
  cfgpath = absbuf;
  mkdir(outdir.c_str(), 0755);
  if (chdir(outdir.c_str()) != 0) return 2;

  omp_set_num_threads(1);
  randi = new MTRand*[1];
  randi[0] = new MTRand((MTRand::uint32)seed);
  World::ststep = ststep;

  // keep the reference's console chatter out of the harness output
  std::ofstream chatter("reference_stdout.txt");
  std::streambuf* saved = std::cout.rdbuf(chatter.rdbuf());

  libconfig::Config cfg;
  cfg.readFile(cfgpath.c_str());
  const libconfig::Setting& root = cfg.getRoot();
  wc.loadparameter(root);
  Simulation* sim = new Simulation(root);

  Out out(".");
  {
    double a0[3] = {sim->mpcd.a[0], sim->mpcd.a[1], sim->mpcd.a[2]};
    out.put("shift_0", a0, {3});
    double sz[4] = {(double)sim->mpcd.size[0], (double)sim->mpcd.size[1], (double)sim->mpcd.size[2],
                    (double)sim->md_objects.size()};
    out.put("box", sz, {4});
  }
  dump_state(out, *sim, "step0");
  int ok = 1;
  MTRand clone(1u);
  for (int s = 1; s <= nsteps; ++s) {
    std::vector<double> gamma, axis, virt;
    replay_collision(*sim, clone, gamma, axis, virt);
    sim->next_tstep();
    // shift_boxes draws three more values after the collision (mpcd.cpp:249-253)
    clone.randDblExc();
    clone.randDblExc();
    clone.randDblExc();
    if (!same_state(clone, *randi[0])) ok = 0;
    const long nc = (long)gamma.size();
    out.put("gamma_" + std::to_string(s), gamma, {nc});
    out.put("axis_" + std::to_string(s), axis, {nc, 3});
#if defined(SLIP) || defined(NOSLIP)
    out.put("virt_" + std::to_string(s), virt, {nc, 3});
#endif
    double a[3] = {sim->mpcd.a[0], sim->mpcd.a[1], sim->mpcd.a[2]};
    out.put("shift_" + std::to_string(s), a, {3});
    if (std::find(dumps.begin(), dumps.end(), s) != dumps.end())
      dump_state(out, *sim, "step" + std::to_string(s));
    if (std::find(writes.begin(), writes.end(), s) != writes.end()) {
      for (size_t k = 0; k < sim->md_objects.size(); ++k) sim->md_objects[k]->writedata();
      sim->mpcd.debug();
    }
  }
  double okv = ok;
  out.put("replay_ok", &okv, {1});
  std::cout.rdbuf(saved);
  std::cout << (ok ? "replay consistent" : "REPLAY MISMATCH") << std::endl;
  // Simulation's destructor writes checkpoint files into outdir; keep them.
  delete sim;
  return ok ? 0 : 1;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::cerr << "usage: ref_harness kat|gamma|run ...\n";
    return 2;
  }
  std::string mode = argv[1];
  if (mode == "kat") {
    MTRand r((MTRand::uint32)std::strtoul(argv[2], nullptr, 10));
    int count = std::atoi(argv[3]);
    for (int i = 0; i < count; ++i) std::cout << r.randInt() << "\n";
    return 0;
  }
  if (mode == "gamma") {
    omp_set_num_threads(1);
    randi = new MTRand*[1];
    randi[0] = new MTRand((MTRand::uint32)std::strtoul(argv[2], nullptr, 10));
    int nc = std::atoi(argv[3]);
    int count = std::atoi(argv[4]);
    std::cout << std::setprecision(17);
    for (int i = 0; i < count; ++i) std::cout << rgamma(nc) << "\n";
    return 0;
  }
  if (mode == "run") return run_mode(argc, argv);
  std::cerr << "unknown mode\n";
  return 2;
}
