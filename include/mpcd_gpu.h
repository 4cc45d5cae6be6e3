/* mpcd_gpu.h -- C ABI of the GB300 MPCD + microswimmer engine (libmpcd_gpu.so).
 *
 * One handle is one simulation box on one GPU: MPCD fluid particles, MD beads
 * with their spring network, and the per-cell state of the SRD collision.
 * The entry points replace the bodies of the reference's hot path:
 *
 *   mpcd_step           Simulation::next_tstep          (src/simulation.cpp:217-265)
 *                       = MPCD::next_tstep (collision)  (src/libcilia/mpcd.cpp:140-247)
 *                       + n x (md_loop*, recalc_forces) (src/libcilia/mdobject.cpp:36-72,
 *                                                        src/simulation.cpp:202-215)
 *                       + MPCD::shift_boxes             (src/libcilia/mpcd.cpp:249-253)
 *                       + Fluid::move / md_loop_stop    (src/libcilia/fluid.cpp:152-167,
 *                                                        src/libcilia/mpcd.cpp:340-394)
 *                       + switch_logic                  (src/cilia.cpp:241-258,
 *                                                        src/ConstantBeatCilia.cpp:8-23)
 *   mpcd_set_fluid      Fluid::create / Fluid::load then add_impuls (src/libcilia/fluid.cpp:55-98,
 *                       120-150, src/libcilia/mpcd.cpp:257-267)
 *   mpcd_set_beads      MDObject::init (src/libcilia/mdobject.cpp:153-160)
 *   mpcd_set_springs    the spring calls of Cilia::recalcforce/addcross, Sphere::recalcforce and
 *                       Clami::global_forces (src/cilia.cpp:127-239, src/sphere.cpp:87-119,
 *                       src/clami.cpp:188-198), flattened into one list
 *   mpcd_set_cilia      per-cilium beat state (newlength/oldlength/midpnt/Tstroke, src/cilia.h:54-65)
 *   mpcd_observables    MPCD::debug totals (src/libcilia/mpcd.cpp:404-467), Fluid::writedata
 *                       (src/libcilia/fluid.cpp:169-207) and diss_energy_total
 *   mpcd_get_shift /
 *   mpcd_set_shift      MPCD::a, persisted in mpcd.dat (src/libcilia/mpcd.cpp:86-97, 396-403)
 *
 * Conventions: every function returns 0 on success or a positive MPCD_E* code;
 * mpcd_last_error() gives the message.  No exception crosses the boundary.
 * All pointers are HOST pointers; the library copies.  Arrays are row-major
 * float64: positions and velocities are n x 3.  A handle must be used from one
 * host thread at a time; it owns one CUDA stream.
 */
#ifndef MPCD_GPU_H
#define MPCD_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPCD_OK 0
#define MPCD_EINVAL 1   /* bad argument */
#define MPCD_ECUDA 2    /* CUDA runtime error */
#define MPCD_ESTATE 3   /* call out of order (e.g. stepping before set_fluid) */
#define MPCD_EDEVICE 4  /* a device-side check failed (see mpcd_last_error) */
#define MPCD_ENOMEM 5   /* device allocation failed */

/* arithmetic of the fluid path */
#define MPCD_FP64 0 /* plain: int cell + float64 in-cell offset, float64 velocities */
#define MPCD_FP32 1 /* split: int cell + float32 in-cell offset, float32 velocities */

/* boundary conditions along z (compile-time -DNOSLIP / -DSLIP in the reference) */
#define MPCD_WALLS_NONE 0
#define MPCD_WALLS_NOSLIP 1 /* bounce-back + virtual particles (src/libcilia/mpcd.cpp:175-198, 346-376) */
#define MPCD_WALLS_SLIP 2

typedef struct mpcd_engine mpcd_engine;

typedef struct {
  int sizes[3];          /* box edges in collision cells (cell size a = 1), each 2..1024 */
  double tstep;          /* MPC time step h (wc.tstep) */
  double ststep;         /* MD substep (World::ststep); substeps n = int((h + 1e-8) / ststep) */
  int precision;         /* MPCD_FP64 or MPCD_FP32 */
  int walls;             /* MPCD_WALLS_* */
  double gravity;        /* body-force amplitude along x (FLUID_FLOW_G); 0 = off */
  double omega;          /* body force ~ gravity * cos(omega * t) (src/libcilia/fluid.cpp:156-158) */
  double bead_mass;      /* collision mass of MD beads (MDObject::partmass = 5) */
  unsigned long long seed; /* counter-based generator seed for free-running steps */
  int device;            /* CUDA device ordinal */
  int sort_interval;     /* reorder particles by cell every this many steps (0 = auto: 50) */
  int md_split;          /* MD arithmetic: -1 auto (2 for MPCD_FP64, 3 for MPCD_FP32),
                            0 float64, 1 split (float springs on hi/lo position pairs; state
                            stays float64), 2 double-float (pairs of floats, about 48
                            significand bits, for forces and substeps; float64 between steps),
                            3 float springs (split arithmetic) on the layout of 2,
                            4 float64 with each spring and its reverse evaluated once and a
                            sphere centre's force summed from its partners' reactions
                            (faster than 0 on GB300), 5 the same in double-float */
} mpcd_params;

/* Values that replace the generator for one step (all host arrays).  Used to
 * reproduce a run of the reference exactly: the grid shift drawn after the
 * collision, and for every cell the Gamma variate (rgamma, used only when the
 * cell holds more than one particle and positive relative kinetic energy) and
 * the unit rotation axis. */
typedef struct {
  const double* shift_next; /* [3], in (0,1): MPCD::a after shift_boxes */
  const double* gamma;      /* [ncells]; < 0 where the reference drew none */
  const double* axis;       /* [ncells][3] */
  const double* virt;       /* [ncells][3] virtual-particle momentum of the wall-layer cells
                               (src/libcilia/mpcd.cpp:175-198); NULL: from the generator */
} mpcd_inject;

typedef struct {
  double momentum[3];  /* total momentum / total mass, fluid + beads */
  double n;            /* particles counted (fluid + beads) */
  double mass;         /* total mass */
  double kT;           /* sum m v^2 / (3 N) over fluid + beads (mpcd.san) */
  double fluid_T;      /* sum v^2 / (3 N_fluid) over fluid (temp.san) */
  double diss_energy;  /* MPCD::diss_energy_total since the last reset */
  double globalt;      /* simulation time */
  double energy_fluid; /* sum m v^2 / 2 over fluid, float64 */
} mpcd_obs;

/* lifecycle */
int mpcd_create(const mpcd_params* params, mpcd_engine** out);
int mpcd_destroy(mpcd_engine* h);
const char* mpcd_last_error(const mpcd_engine* h);
long mpcd_cell_count(const mpcd_engine* h);

/* fluid (mass 1): n x 3 positions (any periodic image) and velocities */
int mpcd_set_fluid(mpcd_engine* h, long n, const double* pos, const double* vel);
/* positions come back wrapped into [0, L) */
int mpcd_get_fluid(mpcd_engine* h, long n, double* pos, double* vel);
long mpcd_fluid_count(const mpcd_engine* h);
/* Page-lock (and release) a caller's host buffer, e.g. the arrays given to
 * mpcd_set_fluid / mpcd_get_fluid, so that their copies run as direct DMA
 * rather than through staging of pageable memory; unpin before freeing it. */
int mpcd_pin_host(mpcd_engine* h, void* p, size_t bytes);
int mpcd_unpin_host(mpcd_engine* h, void* p);

/* grid shift and simulation time */
int mpcd_set_shift(mpcd_engine* h, const double* a3);
int mpcd_get_shift(mpcd_engine* h, double* a3);
int mpcd_set_time(mpcd_engine* h, double globalt);
int mpcd_get_time(mpcd_engine* h, double* globalt);

/* MD beads, in md_objects order (rod-major).  moves[i] = 0 for beads below an
 * object's startidx: they exert forces but are neither integrated nor binned. */
int mpcd_set_beads(mpcd_engine* h, long nb, const double* pos, const double* vel, const int* moves);
int mpcd_get_beads(mpcd_engine* h, long nb, double* pos, double* vel);

/* Spring kinds.  Every entry is one-sided: the force acts on `target` only,
 * F = -2 k (1 - b / |d|) d with d = x_target - x_other (MDObject::spring,
 * src/libcilia/mdobject.cpp:8-17).  The rest length b is
 *   MPCD_SPRING_CONST   : rest[i]
 *   MPCD_SPRING_GUARDED : rest[i], and F = 0 when |d| == 0 (vector form, mdobject.cpp:19-29)
 *   MPCD_SPRING_BOND    : newlength[ref[i]] of the cilium bond table
 *   MPCD_SPRING_DIAG    : sqrt(0.5^2 + 0.5 * newlength[ref[i]]) (cilia.cpp:153, 179)
 * A bead sums its springs in list order, as the reference does. */
#define MPCD_SPRING_CONST 0
#define MPCD_SPRING_GUARDED 1
#define MPCD_SPRING_BOND 2
#define MPCD_SPRING_DIAG 3
int mpcd_set_springs(mpcd_engine* h, long ns, const int* target, const int* other, const int* kind,
                     const int* ref, const double* rest, const double* k);

/* Cilia with an active beat (Cilia / ConstantBeatCilia).  bond_base indexes the
 * newlength/oldlength tables (rodlength entries per cilium). */
#define MPCD_CILIUM_BASIC 0    /* Cilia::switch_logic (curvature-triggered) */
#define MPCD_CILIUM_CONSTANT 1 /* ConstantBeatCilia::switch_logic (time-driven) */
typedef struct {
  int kind;
  int rodlength;
  int num_anker;
  int bead0;     /* bead index of (filament 0, bead 0); filaments f at bead0 + f*rodlength */
  int bond_base; /* first entry of this cilium in the newlength/oldlength tables */
  double beatstrength, bending, max_bend, m_speed;
  double power_stroke_duration, recovery_stroke_duration;
  double start;   /* = num_anker */
  double midpnt;  /* beat state */
  double tstroke; /* Tstroke */
} mpcd_cilium;
/* newlength/oldlength: the bond tables (sum of rodlength entries) */
int mpcd_set_cilia(mpcd_engine* h, int nc, const mpcd_cilium* cilia, const double* newlength,
                   const double* oldlength);
/* out: per cilium [midpnt, tstroke]; newlength/oldlength tables may be NULL */
int mpcd_get_cilia(mpcd_engine* h, int nc, double* state2, double* newlength, double* oldlength);

/* bins fluid and beads with the current shift (end of Simulation's constructor) */
int mpcd_prepare(mpcd_engine* h);

/* one MPC step; inj may be NULL (counter-based generator) */
int mpcd_step(mpcd_engine* h, const mpcd_inject* inj);
/* nsteps free-running MPC steps; observables read back only at the end */
int mpcd_run(mpcd_engine* h, int nsteps);
int mpcd_observables(mpcd_engine* h, mpcd_obs* out);
/* The same observables without stalling the host: mpcd_observables_async
 * enqueues the sums of the current state on the handle's stream and returns a
 * ticket at once; mpcd_observables_result waits for that ticket's read-back
 * only (not for steps issued after it) and fills out as mpcd_observables does,
 * globalt included.  The newest MPCD_OBS_RING tickets can be collected, in any
 * order and more than once; an older or never-issued ticket is MPCD_EINVAL.
 * No counterpart in the reference (MPCD::debug prints at once). */
#define MPCD_OBS_RING 256
int mpcd_observables_async(mpcd_engine* h, long long* ticket);
int mpcd_observables_result(mpcd_engine* h, long long ticket, mpcd_obs* out);
int mpcd_reset_diss(mpcd_engine* h);
/* waits for the handle's stream; reports device-side errors */
int mpcd_sync(mpcd_engine* h);

/* kernel launches issued by this handle so far (for accounting) */
long long mpcd_launch_count(const mpcd_engine* h);

/* Timing on the handle's stream.  Runs nsteps free-running steps, each
 * bracketed by CUDA events; with flush_l2 != 0 a 256 MB scratch buffer is
 * written between steps (outside the timed pairs) so that every step starts
 * with a cold L2.  step_ms (may be NULL) receives each step's device time. */
int mpcd_timed_run(mpcd_engine* h, int nsteps, int flush_l2, double* step_ms);

/* Per-kernel device times: with profiling on, every launch is bracketed by
 * events.  kernel: MPCD_K_* ; returns total milliseconds and launch count
 * since profiling was switched on. */
#define MPCD_K_CELL 0   /* cell_params: collision maps */
#define MPCD_K_FLUID 1  /* fluid_step: collide + stream + bin */
#define MPCD_K_BEAD 2   /* bead_collide */
#define MPCD_K_MD 3     /* md: all substeps */
#define MPCD_K_SORT 4   /* counting-sort reorder */
int mpcd_set_profiling(mpcd_engine* h, int on);
int mpcd_kernel_time(mpcd_engine* h, int kernel, double* total_ms, long long* launches);

/* Layout the MD kernels run on (built first if the bead set changed).
 * info[8] receives: cluster (1: one thread-block cluster, 0: cooperative
 * grid), threads per slot, slots per tile, tiles (CTAs), slots, springs,
 * largest halo of a tile, arithmetic (0 float64, 1 split, 2 double-float,
 * 3 float springs on the double-float layout, 4 float64 pair kernel, 5
 * double-float pair kernel; for 4 and 5 "threads per slot" is the CTA's
 * threads over its slots, and springs excludes the dropped lists of sphere
 * centres). */
int mpcd_md_layout(mpcd_engine* h, int* info);

/* Lossless snapshots of a handle's whole state, for checkpoints that keep
 * every bit (the reference's own checkpoint files, which `cilia` writes and
 * reads as well, round the fluid to 7 digits: src/libcilia/fluid.cpp:100-108)
 * and for moving a run between handles: fluid in the engine's own layout,
 * beads, springs, cilia and their beat state, grid shift, time, step counter
 * and generator seed, dissipated energy, rigid spheres.  mpcd_snapshot_size
 * gives the bytes; mpcd_snapshot fills a host buffer of at least that size;
 * mpcd_restore loads one into a handle created with the same box, precision,
 * tstep and ststep (MPCD_EINVAL otherwise) and replaces its state.  The first
 * step after a restore bins the particles again, so a restored run continues
 * the original one to the order of floating-point additions into cell sums. */
int mpcd_snapshot_size(mpcd_engine* h, long long* bytes);
int mpcd_snapshot(mpcd_engine* h, void* buf, long long bytes);
int mpcd_restore(mpcd_engine* h, const void* buf, long long bytes);

/* ----------------------------------------------------------------------------
 * Rigid spheres with no-slip bounce-back.  The reference's bounce-back
 * surfaces are the planar walls of -DNOSLIP (streaming reflection,
 * src/libcilia/mpcd.cpp:346-376; virtual particles in the wall layers,
 * mpcd.cpp:175-198); these calls extend the same two rules to spheres, an
 * addition with no counterpart in the reference's object model (its Sphere is
 * a bead-spring mesh coupled through the collision only):
 *   - streaming: a fluid particle that reaches a sphere's surface during the
 *     step leaves the contact point with v' = 2 u_s - v, u_s the surface
 *     velocity V + W x r_c, for the rest of the step;
 *   - collision: a cell the surface cuts that holds n < 10 particles gets
 *     10 - n virtual particles moving with u_s at the cell centre plus
 *     thermal noise at kT = 1 (or the injected mpcd_inject.virt);
 *   - both exchanges are summed per sphere in float64 (impulse and angular
 *     impulse); a free sphere (mass > 0, solid: I = 2/5 m r^2) takes them into
 *     its velocity and angular velocity after every step and moves with its
 *     velocity; a held sphere (mass <= 0) keeps its velocity and angular
 *     velocity (0 for a fixed obstacle).
 * Spheres smaller than half the box have periodic images; larger ones (a
 * sphere of very large radius stands for a curved wall) have none.  Fluid
 * should be placed outside the spheres: a particle found inside at the start
 * of a step is put on the surface and reflected there.  At most
 * MPCD_MAX_RIGID_SPHERES; n = 0 removes them.  The getter returns the state
 * and, in force_torque[n][6] (may be NULL), the mean force and torque the
 * fluid exerted since the spheres were set or the sums reset.
 * -------------------------------------------------------------------------- */
#define MPCD_MAX_RIGID_SPHERES 4
typedef struct {
  double center[3];
  double velocity[3];
  double omega[3];
  double radius;
  double mass; /* > 0 free, <= 0 held */
} mpcd_rigid_sphere;
int mpcd_set_rigid_spheres(mpcd_engine* h, int n, const mpcd_rigid_sphere* spheres);
int mpcd_get_rigid_spheres(mpcd_engine* h, int n, mpcd_rigid_sphere* spheres, double* force_torque);
int mpcd_reset_rigid_sphere_forces(mpcd_engine* h);
int mpcd_rigid_sphere_count(const mpcd_engine* h);

/* Contact forces between cilia: GlobalForces::recalc_forces / vdw_force of
 * the reference built with -DREPELLING=eps (src/libcilia/globalforces.cpp:
 * 22-95; cutoff 1.5, stride N = 4): a harmonic repulsion of the section
 * centroids of two cilia closer than the cutoff, F = -2 eps (1 - 1.5 / |d|) d,
 * added to the three beads of each section, in every MD force evaluation,
 * over the cilia in mpcd_set_cilia order.  (The reference's own code for it
 * does not compile: it names a `cilias` list that its class does not
 * declare.)  eps = 0 turns it off.  With eps != 0 the MD substeps run on the
 * float64 grid kernel, whatever mpcd_params.md_split says; cilia of at most 64
 * beads per filament. */
int mpcd_set_repelling(mpcd_engine* h, double eps);

/* The counter-based generator's collision draws, for checking them against
 * the reference's samplers: for cells k = 0 .. n-1 of step `step` under
 * `seed`, gamma[k] is the Gamma(3(nc-1)/2, 1) variate a free-running step
 * gives a cell of nc particles (rgamma, src/libcilia/mpcd.cpp:13-43) and
 * axis[3k..3k+2] the float64 path's unit rotation axis
 * (generate_collision_matrix, src/libcilia/mpcd.cpp:269-284).  Host arrays;
 * either may be NULL.  Runs on `device` (allocates and frees its own device
 * buffers).  MPCD_EDEVICE when a Gamma draw hit the sampler's iteration cap. */
int mpcd_collision_draws(int nc, unsigned long long seed, unsigned long long step, long n, double* gamma,
                         double* axis, int device);

/* ----------------------------------------------------------------------------
 * mpcd_fluid_step_noalloc -- one split-precision MPC step of a plain fluid
 * (collision, streaming, binning; no beads, no walls) that allocates no device
 * memory.  It has no counterpart in the reference: it exists for callers that
 * cannot call cudaMalloc themselves -- code that runs inside another runtime's
 * memory pool or allocator, or a plug-in that is only handed device pointers
 * and a stream.
 *
 * The caller passes the particles in device-accessible memory, in the engine's
 * split layout, and gets them back in place:
 *   pos[i] = float4(ox, oy, oz, c) with in-cell offsets in [0,1) and c the
 *            bits of the uint32 cell index ix | iy << 10 | iz << 20
 *   vel[i] = float4(vx, vy, vz, 0)
 * On entry the particles are binned with the grid shift a_cur; the step
 * collides them (thermostat and rotation axis from the counter-based generator
 * at (seed, step), as mpcd_step draws them), streams them by tstep and leaves
 * them for a next call with a_cur = a_next.  diss (host, may be NULL) receives
 * the kinetic energy removed by the thermostat.  stream: a cudaStream_t (NULL
 * for the default stream); the call returns after the stream has finished.
 *
 * Its per-cell scratch is a file-scope static device array for at most
 * MPCD_NOALLOC_MAX_CELLS cells (about 3.4 MB), held by every GPU that loads the
 * library until the process exits.  Larger boxes are rejected with
 * MPCD_EINVAL.  The first call on a device looks the array's address up
 * (cudaGetSymbolAddress) with that device current.  Every call synchronizes
 * `stream` (it reads the layout check, the error word and the dissipated
 * energy back), so it must not be called on a stream that is being captured.
 * All calls share the array: calls that overlap on the GPU race, and the
 * array keeps the last call's contents.  Particles that break the layout
 * above (a cell index at or beyond its box edge, an offset outside [0,1)) are
 * rejected with MPCD_EDEVICE before anything is changed.
 * Returns MPCD_OK, MPCD_EINVAL, MPCD_ECUDA, or MPCD_EDEVICE (a device-side check failed).
 * -------------------------------------------------------------------------- */
#define MPCD_NOALLOC_MAX_CELLS 65536
int mpcd_fluid_step_noalloc(const int* sizes, long n, void* pos, void* vel, double tstep, const double* a_cur,
                            const double* a_next, unsigned long long seed, unsigned long long step, double* diss,
                            void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MPCD_GPU_H */
