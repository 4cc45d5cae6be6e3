// Host object model of the microswimmer simulation, mirroring the reference's
// classes (src/libcilia/mdobject.h, src/sphere.h, src/cilia.h,
// src/ConstantBeatCilia.h, src/clami.h, src/simulation.h).  The objects own the
// geometry and the topology; the numerics run on the GPU through mpcd_gpu.h.
// Each object turns its spring calls into entries of one flat spring list, in
// the order the reference calls them, so that every bead sums its forces in
// the reference's order.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "libconfig_lite.hpp"
#include "mpcd_batch.h"
#include "mpcd_gpu.h"

namespace cilia {

// Flat spring list handed to mpcd_set_springs.
struct SpringList {
  std::vector<int> target, other, kind, ref;
  std::vector<double> rest, k;
  void add(long t, long o, int kd, int rf, double b, double kk) {
    target.push_back((int)t);
    other.push_back((int)o);
    kind.push_back(kd);
    ref.push_back(rf);
    rest.push_back(b);
    k.push_back(kk);
  }
  size_t size() const { return target.size(); }
};

// MT19937 as used through the reference's MTRand (src/libcilia/MersenneTwister.h):
// rnd() = randDblExc, normalrand() = Box-Muller cosine branch (src/libcilia/basicf.h).
class HostRng {
 public:
  explicit HostRng(uint32_t seed) : mt_(seed) {}
  double rnd() { return ((double)mt_() + 0.5) * (1.0 / 4294967296.0); }
  double normalrand() {
    double x1 = rnd(), x2 = rnd();
    return std::sqrt(-2.0 * std::log(x1)) * std::cos(2.0 * 3.14159265358979323846 * x2);
  }
  uint32_t u32() { return (uint32_t)mt_(); }

 private:
  std::mt19937 mt_;
};

class MDObject {
 public:
  MDObject(std::string name, int num_rods, int rodlength, int startidx = 0, bool write_data = true)
      : name(std::move(name)), num_rods(num_rods), rodlength(rodlength), startidx(startidx),
        write_data(write_data), pos((size_t)num_rods * rodlength * 3, 0.0), vel((size_t)num_rods * rodlength * 3, 0.0) {}
  virtual ~MDObject() = default;

  std::string name;
  int num_rods, rodlength, startidx;
  bool write_data;
  std::vector<double> pos, vel;  // [rod][bead][3]
  long bead_offset = 0;          // global index of (rod 0, bead 0)
  bool loaded = false;

  long nbeads() const { return (long)num_rods * rodlength; }
  double* P(int r, int j) { return &pos[3 * ((size_t)r * rodlength + j)]; }
  const double* P(int r, int j) const { return &pos[3 * ((size_t)r * rodlength + j)]; }
  long bead(int r, int j) const { return bead_offset + (long)r * rodlength + j; }

  // recalcforce / global_forces as flat spring entries
  virtual void emit_forces(SpringList&) const {}
  virtual void emit_global_forces(SpringList&) const {}
  virtual void emit_cilia(std::vector<mpcd_cilium>&, std::vector<double>&, std::vector<double>&) const {}
  virtual void take_cilia_state(const double*, const double*, const double*) {}
  virtual const char* type_name() const = 0;
  // output (MDObject::writedata, src/libcilia/mdobject.cpp:83-107) and checkpoint
  virtual void writedata(double globalt);
  virtual void save(std::ostream& out) const;
  void save() const;
  virtual bool load(std::istream& in);
  bool open_datfile();
  // whether constructors read <name>.dat checkpoints (set by the Simulation)
  static thread_local bool read_files;
};

class Sphere : public MDObject {
 public:
  Sphere(const libconfig::Setting& cfg);
  Sphere(double radius, double springconstant, double wx, double wy, double wz, int npart, std::string name,
         bool write = true);
  double springconstant, radius, headbond = 0.0;
  int npart;
  std::vector<std::array<int, 7>> neilist;
  void emit_forces(SpringList& s) const override;
  const char* type_name() const override { return "Sphere"; }
  void save(std::ostream& out) const override;
  bool load(std::istream& in) override;

 private:
  void create(double wx, double wy, double wz, int fill);
  void create_neillist(int max_part);
};

class Cilia : public MDObject {
 public:
  Cilia(const libconfig::Setting& cfg);
  Cilia(const libconfig::Setting& cfg, const double* pos3, double thetaX, double thetaY, double thetaZ,
        std::string name, int startidx, int num_anker);
  double beatstrength = 0, bending = 0, min_bend = 0, max_bend = 0, m_speed = 1, springconstant = 0;
  int num_anker = 0;
  int bond_base_ = 0;  // first entry of this cilium in the engine's bond tables
  double start, midpnt, Tstroke = 0.0;
  std::vector<double> newlength, oldlength;
  virtual int beat_kind() const { return MPCD_CILIUM_BASIC; }
  virtual double power_dur() const { return 0.0; }
  virtual double recovery_dur() const { return 0.0; }
  void emit_forces(SpringList& s) const override;
  void emit_cilia(std::vector<mpcd_cilium>& c, std::vector<double>& nl, std::vector<double>& ol) const override;
  void take_cilia_state(const double* st2, const double* nl, const double* ol) override;
  const char* type_name() const override { return "Cilia"; }
  void save(std::ostream& out) const override;
  bool load(std::istream& in) override;

 protected:
  void init(const libconfig::Setting& cfg, double wx, double wy, double wz, double tx, double ty, double tz);
  void create(double wx, double wy, double wz, double thetaX, double thetaY, double thetaZ);
};

class ConstantBeatCilia : public Cilia {
 public:
  ConstantBeatCilia(const libconfig::Setting& cfg);
  ConstantBeatCilia(const libconfig::Setting& cfg, const double* pos3, double tx, double ty, double tz,
                    std::string name, int startidx, int num_anker);
  double power_stroke_duration, recovery_stroke_duration;
  int beat_kind() const override { return MPCD_CILIUM_CONSTANT; }
  double power_dur() const override { return power_stroke_duration; }
  double recovery_dur() const override { return recovery_stroke_duration; }
  const char* type_name() const override { return "ConstantBeatCilia"; }
};

class Simulation;

class Clami : public MDObject {
 public:
  Clami(const libconfig::Setting& cfg, Simulation& sim);
  struct Attach {
    int cil;      // index into cilias
    int sphere_bead, rod, bead;
    double l0;
  };
  double springconstant = 20000.0;
  Sphere* sphere = nullptr;
  std::vector<Cilia*> cilias;
  std::vector<Attach> springs;
  long num_particles = 0;
  void emit_global_forces(SpringList& s) const override;
  const char* type_name() const override { return "Clami"; }
  void writedata(double globalt) override;
  void save(std::ostream& out) const override;
  bool load(std::istream& in) override;
  double diss_energy_interval = 0.0;  // set by the simulation before writedata
  double tstep = 0.1;
  int measureinterval = 50;

 private:
  void attach(Cilia* c, int cidx, int wo);
};

struct World {
  double globalt = 0.0, desiredt = 0.0, runtime = 0.0, omega = 0.0, tstep = 0.1, ststep = 0.001;
  int sizex = 100, sizey = 100, sizez = 50;
  int measureinterval = 50;
  void loadparameter(const libconfig::Setting& root);
  void saveparameter(libconfig::Setting& root) const;
};

struct SimOptions {
  int precision = MPCD_FP64;
  int device = 0;
  uint64_t seed = 0;       // 0: from the cfg `seed` key, else /dev/urandom
  double ststep = 0.0;     // > 0 overrides the cfg/default MD step
  int create_fluid = 1;    // 0: leave the fluid empty (set it through the engine)
  int read_files = 1;      // load <name>.dat / fluid_n.dat / mpcd.dat when present
  int walls = MPCD_WALLS_NONE;
  double gravity = 0.0;
  double bead_mass = 5.0;
  int sort_interval = 0;
  int md_split = -1;       // -1 auto, 0 float64 springs, 1 split springs
  int host_only = 0;       // 1: no engine; the system is only described on the host (HostSystem)
};

// Everything the engine would receive, kept on the host (host_only runs):
// the input of a replica batch (mpcd_batch.h).
struct HostSystem {
  mpcd_params p{};
  double a[3] = {0.5, 0.5, 0.5};
  double globalt = 0.0;
  std::vector<double> fpos, fvel;  // fluid, n x 3
  std::vector<double> bpos, bvel;  // beads, nb x 3
  std::vector<int> moves;
  SpringList springs;
  std::vector<mpcd_cilium> cilia;
  std::vector<double> newlen, oldlen;
};

// Adds a host-described system to a replica batch as a new replica (not yet
// admitted); throws std::runtime_error with the batch's message on failure.
void add_to_batch(mpcd_batch* b, const HostSystem& h, long nbeads, int* replica);

class Simulation {
 public:
  Simulation(const libconfig::Setting& root, const SimOptions& opt);
  ~Simulation();
  Simulation(const Simulation&) = delete;
  Simulation& operator=(const Simulation&) = delete;

  World wc;
  SimOptions opt;
  uint64_t seed = 0;
  std::unique_ptr<HostRng> rng;
  std::vector<std::unique_ptr<MDObject>> md_objects;
  mpcd_engine* eng = nullptr;
  HostSystem host;  // host_only: what the engine would have received
  long nbeads = 0;

  MDObject* add_md_object(const libconfig::Setting& cfg);
  void write_measure(bool objects, bool debug_row);
  void add_md_object(MDObject* obj);  // takes ownership
  void upload_md();                  // beads + springs + cilia to the engine
  void sync_from_device();           // bead state back into the objects
  int next_tstep(const mpcd_inject* inj = nullptr);
  void run();
  void save_all() const;
  void debug(const char* path);      // MPCD::debug line in mpcd.san
  void write_fluid_temp(const char* path);

 private:
  void create_fluid();
  bool load_fluid(const char* path);
  void save_fluid(const char* path) const;
};

}  // namespace cilia
