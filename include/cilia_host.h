/* cilia_host.h -- C ABI of the simulation driver (libmpcd_gpu.so).
 *
 * A cilia_sim is the reference's Simulation (src/simulation.h:13-48) built
 * from a sim.cfg: the MPCD box, the md_objects (Sphere, Cilia,
 * ConstantBeatCilia, Clami) and the fluid, with the numerics on the GPU
 * engine of mpcd_gpu.h.  It is what `cilia sim.cfg` runs, exposed for callers
 * that drive it step by step (Python through ctypes, other languages through
 * their FFI).
 *
 *   cilia_sim_create     Simulation::Simulation(const Setting&) (src/simulation.cpp:19-35)
 *   cilia_sim_next_tstep Simulation::next_tstep (src/simulation.cpp:217-265)
 *   cilia_sim_run        Simulation::run (src/simulation.cpp:59-156)
 *   cilia_sim_save       Simulation::~Simulation checkpoint writes (src/simulation.cpp:354-380)
 *
 * Errors: nonzero return (MPCD_E* codes of mpcd_gpu.h); cilia_sim_last_error
 * gives the message (configuration errors carry the libconfig setting path).
 */
#ifndef CILIA_HOST_H
#define CILIA_HOST_H

#include "mpcd_batch.h"
#include "mpcd_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cilia_sim cilia_sim;

typedef struct {
  int precision;           /* MPCD_FP64 or MPCD_FP32 */
  int device;              /* CUDA device */
  unsigned long long seed; /* 0: cfg key `seed`, else random */
  double ststep;           /* > 0 overrides the MD step (default: cfg key `ststep`, else 0.001) */
  int create_fluid;        /* 1: create (or load fluid_n.dat); 0: empty, set through the engine */
  int read_files;          /* 1: load <name>.dat, fluid_n.dat, mpcd.dat from the working directory */
  int walls;               /* MPCD_WALLS_* */
  double gravity;          /* body force along x */
  double bead_mass;        /* collision mass of beads (0 = reference value 5) */
  int sort_interval;       /* 0 = default */
  int md_arith;            /* MD arithmetic: 0 auto (double-float for float64, float springs on
                              double-float positions for float32), else mpcd_params.md_split + 1
                              (1 float64, 2 split, 3 double-float, 4 float springs on the
                              double-float layout, 5 float64 pair kernel, 6 double-float pair
                              kernel) */
} cilia_options;

/* cfg is a file path, or libconfig text when is_text != 0 */
int cilia_sim_create(const char* cfg, int is_text, const cilia_options* opt, cilia_sim** out);
int cilia_sim_destroy(cilia_sim* s);
const char* cilia_sim_last_error(const cilia_sim* s);
mpcd_engine* cilia_sim_engine(cilia_sim* s);

int cilia_sim_num_objects(const cilia_sim* s);
/* info[0..4] = rods, rodlength, startidx, bead offset, type (0 Sphere, 1 Cilia, 2 ConstantBeatCilia, 3 Clami) */
int cilia_sim_object_info(const cilia_sim* s, int obj, int* info5, char* name, int name_len);
long cilia_sim_bead_count(const cilia_sim* s);

int cilia_sim_next_tstep(cilia_sim* s, const mpcd_inject* inj);
int cilia_sim_run(cilia_sim* s);
int cilia_sim_save(cilia_sim* s);
/* The writes of Simulation::run after a measure interval (src/simulation.cpp:
 * 103-107), in the working directory: flags bit 0, every object's writedata
 * (Clami::writedata, src/clami.cpp:208-284: <name>.xyz frame and <name>.san
 * row; the dissipated energy is cleared afterwards); bit 1, MPCD::debug's row
 * of mpcd.san (src/libcilia/mpcd.cpp:404-467). */
#define CILIA_WRITE_OBJECTS 1
#define CILIA_WRITE_DEBUG 2
int cilia_sim_writedata(cilia_sim* s, int flags);
/* Builds the system a sim.cfg describes on the host only (objects, springs,
 * cilia, the fluid of Fluid::create or fluid_n.dat, the grid shift) and adds
 * it to a replica batch as a new replica, not yet admitted (mpcd_batch_admit).
 * opt->precision is ignored: a batch runs MPCD_FP32.  Errors from the cfg
 * come back through cilia_sim_last_error(NULL), from the batch through
 * mpcd_batch_last_error. */
int cilia_batch_add_cfg(mpcd_batch* b, const char* cfg, int is_text, const cilia_options* opt, int* replica);
/* writes the cfg back with the current globalt (src/main.cpp:95-96) */
int cilia_sim_write_cfg(cilia_sim* s, const char* path);
/* The initial state the Simulation's constructor (src/simulation.cpp:19-35)
 * builds from a sim.cfg, on the host only and without a GPU: the grid shift
 * (MPCD::MPCD), the md_objects' beads (Sphere::create, Cilia::create,
 * Clami::attach) and, with opt->create_fluid, the fluid of Fluid::create
 * (src/libcilia/fluid.cpp:55-98) or fluid_n.dat.  sizes = {fluid particles,
 * beads, one-sided springs}: call with every array NULL to get them, then
 * with arrays of those sizes (n x 3 each; any may stay NULL).  Errors come
 * back through cilia_sim_last_error(NULL). */
int cilia_cfg_host_state(const char* cfg, int is_text, const cilia_options* opt, long sizes[3], double* shift3,
                         double* fluid_pos, double* fluid_vel, double* bead_pos, double* bead_vel);

#ifdef __cplusplus
}
#endif
#endif
