/* CPU oracle for the MPCD + microswimmer hot path (test infrastructure).
 *
 * A plain-C restatement of the reference's algorithm for
 * Simulation::next_tstep (src/simulation.cpp:217-265): SRD collision with the
 * cell-level Maxwell-Boltzmann-scaling thermostat (src/libcilia/mpcd.cpp:140-247),
 * velocity-Verlet MD substeps (src/libcilia/mdobject.cpp:36-72) with the spring
 * forces of Sphere, Cilia, ConstantBeatCilia and Clami, random grid shift and
 * streaming/binning.  Only the tests, the smoke check and bench.py's CPU
 * baseline use it: it is the checker, never the product.
 *
 * Parity is pinned against the reference itself: tests/golden holds fixtures
 * produced by oracle/_ref/ref_harness (the reference's own translation units),
 * and the tests check this restatement against them.
 */
#ifndef MPCD_ORACLE_H
#define MPCD_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sim orc_sim;

/* box edges in cells, MPC step h, MD step, MT19937 seed (MTRand(seed)) */
orc_sim* orc_create(int lx, int ly, int lz, double tstep, double ststep, unsigned int seed);
void orc_destroy(orc_sim* s);

/* generator access (src/libcilia/MersenneTwister.h, src/libcilia/basicf.h:18-62) */
unsigned int orc_mt_next(orc_sim* s);
double orc_rgamma(orc_sim* s, int nc);

/* MPCD construction: draws the initial grid shift (src/libcilia/mpcd.cpp:92-95) */
void orc_init_shift(orc_sim* s);
void orc_set_shift(orc_sim* s, const double* a3);
void orc_get_shift(const orc_sim* s, double* a3);
void orc_set_globalt(orc_sim* s, double t);
double orc_get_globalt(const orc_sim* s);

/* fluid: create with the reference's draws (src/libcilia/fluid.cpp:55-98) or set */
void orc_fluid_create(orc_sim* s);
int orc_fluid_set(orc_sim* s, long n, const double* pos, const double* vel);
long orc_fluid_count(const orc_sim* s);
void orc_fluid_get(const orc_sim* s, double* pos, double* vel);

/* MD objects; each returns the object index (md_objects order) or -1 */
int orc_add_sphere(orc_sim* s, double radius, double k, double x, double y, double z, int npart);
/* kind: 0 = Cilia, 1 = ConstantBeatCilia */
int orc_add_cilia(orc_sim* s, int kind, int rodlength, double beatstrength, double bending,
                  double min_bend, double max_bend, double m_speed, double k, double x, double y,
                  double z, double thetax, double thetay, double thetaz, int startidx, int num_anker,
                  double power_dur, double recovery_dur, double start_delay);
/* Clami composite: sphere(643) + ring-placed cilia + attachment springs.
 * cil_* describe the `cilia` group (kind as above); start_delays may be NULL. */
int orc_add_clami(orc_sim* s, double radius, double k, double x, double y, double z, int nrings,
                  const int* num_eq, const double* y_thetas_deg, const double* theta_offset,
                  const double* start_delays, int cil_kind, int rodlength, double beatstrength,
                  double bending, double min_bend, double max_bend, double m_speed, double cil_k,
                  double thetaz, double power_dur, double recovery_dur);
int orc_num_objects(const orc_sim* s);
/* object info: [kind, rods, len, startidx, bead_offset]; kind 0 sphere, 1 cilia, 2 cbcilia, 3 clami */
void orc_object_info(const orc_sim* s, int obj, int* info5);
long orc_bead_count(const orc_sim* s);
void orc_beads_get(const orc_sim* s, double* pos, double* vel);
int orc_beads_set(orc_sim* s, const double* pos, const double* vel);
/* per-cilium dynamic state: newlength[len], oldlength[len], midpnt, Tstroke */
int orc_cilium_state(const orc_sim* s, int obj, double* out);
double orc_sphere_headbond(const orc_sim* s, int obj);
/* Clami attachment springs: rows of (cilium object, sphere bead, cilia rod, cilia bead, l0) */
int orc_clami_springs(const orc_sim* s, int obj, double* out, int max_rows);

/* bins fluid and beads (bead collision mass 5, src/libcilia/mdobject.cpp:153-160) */
void orc_init_bins(orc_sim* s);

/* One full MPC step.  Each inject pointer may be NULL (draw from MT19937 in the
 * reference's order) or give: shift_next[3], gamma[ncells] (Gamma variate for
 * cells the reference thermostats), axis[ncells*3].  rec_* (may be NULL)
 * receive the values used.  Returns 0, or 1 if an injected gamma is missing
 * for a cell that needs one. */
int orc_step(orc_sim* s, const double* inj_shift_next, const double* inj_gamma,
             const double* inj_axis, double* rec_shift_next, double* rec_gamma, double* rec_axis);
/* the same with walls: inj_virt / rec_virt hold the virtual-particle momentum
 * of every wall-layer cell that took virtual particles ([ncell][3]) */
int orc_step_walls(orc_sim* s, const double* inj_shift_next, const double* inj_gamma, const double* inj_axis,
                   const double* inj_virt, double* rec_shift_next, double* rec_gamma, double* rec_axis,
                   double* rec_virt);
/* boundaries (0 periodic, 1 no-slip, 2 slip walls along z; src/libcilia/mpcd.cpp:175-198,
 * 346-376) and the body force g cos(omega t) along x (src/libcilia/fluid.cpp:156-158) */
void orc_set_walls(orc_sim* s, int walls);
void orc_set_gravity(orc_sim* s, double g, double omega);
/* contact forces between cilia (the reference's -DREPELLING=eps); 0 = off */
void orc_set_repelling(orc_sim* s, double eps);
long orc_contacts(const orc_sim* s);
double orc_diss_energy(const orc_sim* s);
void orc_reset_diss(orc_sim* s);

/* Threads for throughput runs (CPU baseline).  With T > 1 each thread draws from
 * its own MT19937 stream and owns a static block of cells, as the reference's
 * OpenMP build does; results are then not comparable step by step. */
void orc_set_threads(orc_sim* s, int threads);

/* observables: [P_x/M, P_y/M, P_z/M, N, M, kT] over fluid+beads (src/libcilia/mpcd.cpp:404-467) */
void orc_observables(const orc_sim* s, double* out6);

#ifdef __cplusplus
}
#endif
#endif
