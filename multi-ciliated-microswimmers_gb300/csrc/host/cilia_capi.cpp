// C ABI over the host Simulation (include/cilia_host.h).
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>

#include "cilia_host.h"
#include "libconfig_lite.hpp"
#include "objects.hpp"

struct cilia_sim {
  std::unique_ptr<libconfig::Config> cfg;
  std::unique_ptr<cilia::Simulation> sim;
  std::string error;
};

namespace {
thread_local std::string g_create_error;

// translates the reference's error reports (src/main.cpp:56-93) into messages
template <typename F>
int guarded(std::string& err, F f) {
  try {
    return f();
  } catch (const libconfig::ParseException& e) {
    err = std::string("Parse error at ") + e.getFile() + ":" + std::to_string(e.getLine()) + " - " + e.getError();
  } catch (const libconfig::FileIOException&) {
    err = "I/O error while reading file.";
  } catch (const libconfig::SettingNotFoundException& e) {
    err = std::string("No ") + e.getPath() + " setting in configuration file.";
  } catch (const libconfig::SettingTypeException& e) {
    err = std::string("error with:") + e.getPath();
  } catch (const libconfig::SettingException& e) {
    err = std::string("setting error: ") + e.getPath();
  } catch (const std::exception& e) {
    err = e.what();
  }
  return MPCD_EINVAL;
}

cilia::SimOptions to_options(const cilia_options* o) {
  cilia::SimOptions s;
  if (!o) return s;
  s.precision = o->precision;
  s.device = o->device;
  s.seed = o->seed;
  s.ststep = o->ststep;
  s.create_fluid = o->create_fluid;
  s.read_files = o->read_files;
  s.walls = o->walls;
  s.gravity = o->gravity;
  s.bead_mass = o->bead_mass > 0 ? o->bead_mass : 5.0;
  s.sort_interval = o->sort_interval;
  s.md_split = o->md_arith > 0 ? o->md_arith - 1 : -1;
  return s;
}
}  // namespace

extern "C" {

int cilia_batch_add_cfg(mpcd_batch* b, const char* cfg, int is_text, const cilia_options* opt, int* replica) {
  if (!b || !cfg || !replica) return MPCD_EINVAL;
  return guarded(g_create_error, [&]() {
    libconfig::Config c;
    if (is_text)
      c.readString(cfg);
    else
      c.readFile(cfg);
    cilia::SimOptions so = to_options(opt);
    so.host_only = 1;
    so.precision = MPCD_FP32;
    cilia::Simulation sim(c.getRoot(), so);
    cilia::add_to_batch(b, sim.host, sim.nbeads, replica);
    return MPCD_OK;
  });
}

int cilia_cfg_host_state(const char* cfg, int is_text, const cilia_options* opt, long sizes[3], double* shift3,
                         double* fluid_pos, double* fluid_vel, double* bead_pos, double* bead_vel) {
  if (!cfg || !sizes) return MPCD_EINVAL;
  return guarded(g_create_error, [&]() {
    libconfig::Config c;
    if (is_text)
      c.readString(cfg);
    else
      c.readFile(cfg);
    cilia::SimOptions so = to_options(opt);
    so.host_only = 1;
    cilia::Simulation sim(c.getRoot(), so);
    const cilia::HostSystem& h = sim.host;
    const long nf = (long)(h.fpos.size() / 3), nb = (long)(h.bpos.size() / 3);
    // with arrays: they must be the sizes the caller was told
    if ((fluid_pos || fluid_vel || bead_pos || bead_vel) && (sizes[0] != nf || sizes[1] != nb))
      throw std::runtime_error("cilia_cfg_host_state: sizes do not match the system (ask with NULL arrays first)");
    sizes[0] = nf;
    sizes[1] = nb;
    sizes[2] = (long)h.springs.size();
    if (shift3) std::memcpy(shift3, h.a, sizeof h.a);
    if (fluid_pos) std::memcpy(fluid_pos, h.fpos.data(), h.fpos.size() * sizeof(double));
    if (fluid_vel) std::memcpy(fluid_vel, h.fvel.data(), h.fvel.size() * sizeof(double));
    if (bead_pos) std::memcpy(bead_pos, h.bpos.data(), h.bpos.size() * sizeof(double));
    if (bead_vel) std::memcpy(bead_vel, h.bvel.data(), h.bvel.size() * sizeof(double));
    return MPCD_OK;
  });
}

int cilia_sim_create(const char* cfg, int is_text, const cilia_options* opt, cilia_sim** out) {
  if (!cfg || !out) return MPCD_EINVAL;
  *out = nullptr;
  std::unique_ptr<cilia_sim> s(new cilia_sim());
  int rc = guarded(g_create_error, [&]() {
    s->cfg.reset(new libconfig::Config());
    if (is_text)
      s->cfg->readString(cfg);
    else
      s->cfg->readFile(cfg);
    s->sim.reset(new cilia::Simulation(s->cfg->getRoot(), to_options(opt)));
    return MPCD_OK;
  });
  if (rc != MPCD_OK) return rc;
  *out = s.release();
  return MPCD_OK;
}

int cilia_sim_destroy(cilia_sim* s) {
  delete s;
  return MPCD_OK;
}

const char* cilia_sim_last_error(const cilia_sim* s) { return s ? s->error.c_str() : g_create_error.c_str(); }

mpcd_engine* cilia_sim_engine(cilia_sim* s) { return s && s->sim ? s->sim->eng : nullptr; }

int cilia_sim_num_objects(const cilia_sim* s) { return s ? (int)s->sim->md_objects.size() : 0; }

int cilia_sim_object_info(const cilia_sim* s, int obj, int* info5, char* name, int name_len) {
  if (!s || obj < 0 || obj >= (int)s->sim->md_objects.size()) return MPCD_EINVAL;
  const cilia::MDObject* o = s->sim->md_objects[obj].get();
  if (info5) {
    info5[0] = o->num_rods;
    info5[1] = o->rodlength;
    info5[2] = o->startidx;
    info5[3] = (int)o->bead_offset;
    const std::string t = o->type_name();
    info5[4] = t == "Sphere" ? 0 : t == "Cilia" ? 1 : t == "ConstantBeatCilia" ? 2 : 3;
  }
  if (name && name_len > 0) {
    std::strncpy(name, o->name.c_str(), name_len - 1);
    name[name_len - 1] = 0;
  }
  return MPCD_OK;
}

long cilia_sim_bead_count(const cilia_sim* s) { return s ? s->sim->nbeads : 0; }

int cilia_sim_next_tstep(cilia_sim* s, const mpcd_inject* inj) {
  if (!s) return MPCD_EINVAL;
  int rc = s->sim->next_tstep(inj);
  if (rc) s->error = mpcd_last_error(s->sim->eng);
  return rc;
}

int cilia_sim_run(cilia_sim* s) {
  if (!s) return MPCD_EINVAL;
  return guarded(s->error, [&]() {
    s->sim->run();
    return MPCD_OK;
  });
}

int cilia_sim_writedata(cilia_sim* s, int flags) {
  if (!s || flags < 0 || flags > 3) return MPCD_EINVAL;
  return guarded(s->error, [&]() {
    s->sim->write_measure((flags & 1) != 0, (flags & 2) != 0);
    return MPCD_OK;
  });
}

int cilia_sim_save(cilia_sim* s) {
  if (!s) return MPCD_EINVAL;
  return guarded(s->error, [&]() {
    s->sim->sync_from_device();
    s->sim->save_all();
    return MPCD_OK;
  });
}

int cilia_sim_write_cfg(cilia_sim* s, const char* path) {
  if (!s || !path) return MPCD_EINVAL;
  return guarded(s->error, [&]() {
    s->sim->wc.saveparameter(s->cfg->getRoot());
    s->cfg->writeFile(path);
    return MPCD_OK;
  });
}

}  // extern "C"
