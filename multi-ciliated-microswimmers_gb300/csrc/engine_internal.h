// Internal interfaces between the C-ABI host code (engine.cu) and the kernel
// translation units (fluid_kernels.cu, md_kernels.cu).
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "mpcd_device.cuh"

namespace mpcd {

// ---------------------------------------------------------------- fluid ---
// Plain (float64) fluid, structure of arrays.  Position = packed cell +
// in-cell offset in [0,1) per axis.
struct FluidF64 {
  long n = 0;
  uint32_t* id = nullptr;  // caller's index of each particle (permuted by the sort)
  uint32_t* cell = nullptr;
  double *ox = nullptr, *oy = nullptr, *oz = nullptr;
  double *vx = nullptr, *vy = nullptr, *vz = nullptr;
};

// Split-precision fluid: pos = {ox, oy, oz, cell bits}, vel = {vx, vy, vz, 0}.
struct FluidF32 {
  long n = 0;
  uint32_t* id = nullptr;  // caller's index of each particle (permuted by the sort)
  float4* pos = nullptr;
  float4* vel = nullptr;
};

// Per-cell state.  sum: (P_x, P_y, P_z, K) mass-weighted; cnt: fluid count in
// the low 16 bits, bead count in the high 16 bits.  par: collision map
// v' = A v + b, stored as A (row-major 3x3) then b (12 values per cell).
struct CellsF64 {
  long ncell = 0;
  double4* sum = nullptr;
  uint32_t* cnt = nullptr;
  double* par = nullptr;
};
struct CellsF32 {
  long ncell = 0;
  float4* sum = nullptr;
  uint32_t* cnt = nullptr;
  float4* par = nullptr;  // 2 float4 per cell: (axis, thermostat factor), (mean velocity, 0)
};

// Rigid spheres the fluid bounces off (no-slip), with virtual particles in
// the cells their surface cuts.  State on the device, advanced by
// k_spheres_update after every step unless held.
constexpr int kMaxSpheres = 4;
struct RigidSphereDev {
  double c[3];  // centre, in [0, L)
  double v[3];  // velocity
  double w[3];  // angular velocity
  double r;     // radius
  double mass;  // > 0 free; <= 0 held (v, w kept)
  double inertia;
};
struct SphereSet {
  int n = 0;
  const RigidSphereDev* s = nullptr;  // device [n]
  double* acc = nullptr;              // device [n][6]: impulse and angular impulse received this step
};

// Per-step scalars for the fluid kernels.
struct StepArgs {
  Box box;
  double ta_cur[3];   // 1 - a for the shift used by this collision
  double ta_next[3];  // 1 - a for the shift drawn after the MD loop
  double a_cur[3];
  double a_next[3];
  double h;           // MPC time step
  double gkick;       // gravity * cos(omega t) * h, added to v_x after streaming
  int walls;          // MPCD_WALLS_*
  double bead_mass;
  uint64_t seed;
  uint64_t step;      // index of this collision step (generator counter)
  const double* inj_gamma;  // device, or nullptr
  const double* inj_axis;   // device, or nullptr
  const double* inj_virt;   // device [ncell][3] virtual-particle momenta (walls), or nullptr
  unsigned* err;
  double* diss;       // accumulated dissipated energy (float64)
  // float copies for the split-precision kernels (no conversions per thread)
  float fta_cur[3], fta_next[3], fh, fgkick, fbead_mass;
  SphereSet sph;      // rigid spheres (n = 0: none)
  // 1: the maps of the cells holding beads were made by launch_bead_maps
  // this step; the cell-map kernel only clears those cells' sums
  int premapped = 0;
};

// ------------------------------------------------------------------- MD ---
// spring kind flag: the spring's force, negated, is also owed to its other
// bead (a hub whose own list was dropped); only in the cluster layout
constexpr int kSpringReact = 8;
// Spring groups of the cluster layout, the order in which the planner sorts
// every slot's list: CONST, CONST owed to a hub, GUARDED, BOND, DIAG.
__host__ __device__ inline int spring_group(int kraw) {
  const int kind = kraw & 3;
  return kind == 0 ? ((kraw & kSpringReact) ? 1 : 0) : kind + 1;
}
// pair kernel: a bead summing more force entries than this is summed by warps
constexpr int kPairLong = 32;
// pair kernel: a hub (a sphere's centre) that a tile owns or reaches.  The
// hub has no spring list of its own; the tiles holding its partners publish
// the negated sums of their forces, and every tile that reaches it
// integrates a copy from those partial sums.
struct HubRef {
  int hub;     // index into the hub tables
  int idx;     // its staged index in the tile (below the tile size: the tile owns it)
  int rank;    // this tile's partial sum among the hub's contributors, or -1
  int rs, rn;  // incidence slots holding the forces whose reaction the hub takes: tr_list[rs, rs + rn)
  int pad;
};
constexpr int kTileHubs = 4;  // hubs one tile may own or reach
int md_max_coresident_blocks(const struct MDState& m, int f32cells);
int md_cluster_feasible(const struct MDState& m);

struct CiliumDev {
  int kind, len, num_anker, slot0, bond_base;
  int stride;  // slots per bead (every bead of a cilium owns the same number of slots)
  double beatstrength, bending, max_bend, m_speed, power_dur, recovery_dur, start;
};

// Beads live in "slots": the MD kernel runs one thread per slot, a tile of
// slots per CTA, and every cilium lies inside one tile so that its beat
// bookkeeping needs no grid-wide synchronisation.
struct MDState {
  int nslots = 0;        // tiles * tile_size
  int tile = 0;          // threads per CTA
  int ntiles = 0;
  double* x[2] = {nullptr, nullptr};
  double* y[2] = {nullptr, nullptr};
  double* z[2] = {nullptr, nullptr};
  double *vx = nullptr, *vy = nullptr, *vz = nullptr;
  int* moves = nullptr;  // 1 integrated + binned, 0 fixed, 2 helper, -1 empty slot
  int* prim = nullptr;   // helper slot -> primary slot of its bead; primary -> itself
  int* nhelp = nullptr;  // primary slot -> number of helper slots following it
  int* tile_help = nullptr;  // per tile: 1 if it holds helper slots
  int* tile_react = nullptr; // per tile: local slot of a hub fed by reactions, or -1
  // springs in CSR by target slot
  int* sp_start = nullptr;
  int* sp_other = nullptr;
  int* sp_local = nullptr;   // other bead as an index into the tile's staged positions
  int* halo = nullptr;       // per tile: global slots of other tiles' beads its springs reach
  int* halo_start = nullptr; // ntiles + 1
  int hmax = 0;              // largest halo of any tile
  double* diag = nullptr;    // per bond: diagonal rest length sqrt(0.5^2 + 0.5 newlength)
  int split = 0;             // 1: float spring arithmetic on hi/lo position pairs
  int cluster = 0;           // 1: whole bead set in one thread-block cluster (md_cluster.cu)
  int cl_nsp_max = 0;        // cluster layout: most springs of one tile
  int cl_nbond_max = 0;      // cluster layout: most bond-table entries of one tile
  int cl_lanes = 2;          // cluster layout: threads per slot (1 or 2)
  int cl_nbuf = 2;           // cluster layout: position buffers (1 when two do not fit)
  int* sp_kind = nullptr;
  int* sp_ref = nullptr;
  double* sp_rest = nullptr;
  double* sp_m2k = nullptr;  // -2k
  // double-float arithmetic (md_df.cu): float pairs of the spring data,
  // packed spring codes (other bead's staged index | kind << 16 | bond index
  // within the tile << 18), per slot the end of its in-tile springs, per tile
  // its bond range, and two position buffers of pairs, two float4 per slot
  // ({hx, hy, hz, lx}, {ly, lz, 0, 0})
  int df = 0;          // 1: double-float springs, 2: float springs (split arithmetic) on this layout
  int df_nsp_max = 0;  // most springs of one tile
  int df_nb_max = 0;   // most bonds of one tile
  int df_nrun_max = 0;     // most long halo runs of one tile
  int df_nsingle_max = 0;  // most other halo entries of one tile
  float2* sp_rest2 = nullptr;
  float2* sp_m2k2 = nullptr;
  uint32_t* sp_code = nullptr;
  int* sp_split = nullptr;
  int* tile_b0 = nullptr;
  int* tile_nb = nullptr;
  int4* halo_run = nullptr;        // per tile: runs of consecutive halo slots {first, rank, length, 0}
  int* halo_run_start = nullptr;   // ntiles + 1
  int2* halo_single = nullptr;     // per tile: halo entries outside long runs {slot, rank}
  int* halo_single_start = nullptr;
  float4* q[2] = {nullptr, nullptr};
  // pair kernel (md_pair.cu), on the layout above with one slot per bead:
  // per tile its force entries (a spring and its exact reverse inside the
  // tile form one entry; code {a | b << 16, kind | both << 2 | react << 3 |
  // bond << 4}, rest length, -2k, and the incidence slots its force goes to),
  // the entries reaching only the tile's beads first, those reaching a hub
  // last; per slot its range of incidence slots (one per spring of its list,
  // in its spring order); per tile the beads with more than kPairLong
  // incidences.  Positions are published as 32 bytes per slot in q.
  int pair = 0;  // 1 float64, 2 double-float arithmetic
  int pr_nent_max = 0, pr_ninc_max = 0, pr_nlong_max = 0;
  int* pr_start = nullptr;      // ntiles + 1
  int* pr_local_end = nullptr;  // ntiles
  int* pr_hub_begin = nullptr;  // ntiles: entries reaching a hub come last
  uint2* pr_code = nullptr;
  double* pr_rest = nullptr;
  double* pr_m2k = nullptr;
  int* pi_start = nullptr;      // nslots + 1
  uint32_t* pr_pos = nullptr;   // per entry: incidence of its first bead | of its second << 16 (0xffff none)
  int* pl_start = nullptr;      // ntiles + 1
  int* pl_list = nullptr;
  int* pl_base = nullptr;       // each long bead's first incidence slot
  int* pr_nslot = nullptr;      // ntiles: incidence slot words (pr_ninc_max: the most of any tile)
  // hubs: per hub its slot and the offsets of its contributors' partial sums
  // (nhub + 1; hub_ncon in all), two buffers of partial sums (four float64
  // each), per tile its hub references and their entry lists
  int nhub = 0, hub_ncon = 0, ntr = 0;
  int* hub_slot = nullptr;
  int* hub_pbase = nullptr;
  double* hubpart = nullptr;
  int* th_start = nullptr;  // ntiles + 1
  HubRef* th = nullptr;
  int* tr_list = nullptr;
  // cilia
  int ncil = 0;
  CiliumDev* cil = nullptr;
  double* midpnt = nullptr;
  double* tstroke = nullptr;
  double* newlen = nullptr;
  double* oldlen = nullptr;
  int* tile_cil = nullptr;  // ntiles + 1 offsets into cil (cilia sorted by tile)
  GridBarrier bar{nullptr, nullptr};
  // contact forces between cilia (the reference's -DREPELLING=eps, float64 MD
  // kernel only): eps (0 = off), and the cilium pairs whose section bounding
  // boxes came within reach at the start of this MPC step (k_contact_pairs)
  double repel = 0.0;
  int2* cpairs = nullptr;
  int* ncpairs = nullptr;
  int cpair_cap = 0;
};
// candidate cilium pairs of the contact forces for one MPC step (MD stream)
int launch_contact_pairs(const MDState& m, cudaStream_t s);

struct MDStepArgs {
  double t0, dt, tstep;
  double t_end;           // simulation time after the n substeps
  uint64_t refresh[8];    // bit e: force evaluation e (0 .. n) refreshes the beat rest lengths
  int n;
  Box box;
  double a_cur[3], a_next[3];
  double bead_mass;
  unsigned* err;
  // 1: the MD launch first applies the beads' collision (their cells' maps,
  // as the separate bead kernel would) and subtracts their m v'^2 from *diss
  int collide = 0;
  double* diss = nullptr;
  // 1: the beads' final binning goes to bcell / bsum per slot (the cell and
  // its m v, m v^2), added to the cell sums by launch_bead_add after the
  // launch, instead of straight into the cell sums (which the cell-map kernel
  // may still be reading and clearing while the MD runs)
  int deferred = 0;
  uint32_t* bcell = nullptr;
  void* bsum = nullptr;  // double4 per slot (float64 cells) or float4 (split)
};

// ------------------------------------------------------------ launchers ---
// All launchers enqueue on `s` and return the number of kernel launches.
int launch_cell_params_f64(const CellsF64& c, const StepArgs& a, cudaStream_t s);
// per_sm: resident CTAs per SM of the persistent grid (fewer leave room for a concurrent MD launch)
int launch_fluid_step_f64(const FluidF64& f, const CellsF64& c, const StepArgs& a, cudaStream_t s, int per_sm = 4);
int launch_bin_fluid_f64(const FluidF64& f, const CellsF64& c, const StepArgs& a, cudaStream_t s);
int launch_bead_collide_f64(const MDState& m, const CellsF64& c, const StepArgs& a, cudaStream_t s);
int launch_bin_beads_f64(const MDState& m, const CellsF64& c, const StepArgs& a, cudaStream_t s);
int launch_md_f64(const MDState& m, const CellsF64& c, const MDStepArgs& a, cudaStream_t s, cudaError_t* st);
int launch_md_df_f64cells(const MDState& m, const CellsF64& c, const MDStepArgs& a, cudaStream_t s, cudaError_t* st);
int launch_md_df_f32cells(const MDState& m, const CellsF32& c, const MDStepArgs& a, cudaStream_t s, cudaError_t* st);
int md_df_max_coresident_blocks(const MDState& m, int f32cells);
int md_df_lanes(int tile);  // threads per slot of the double-float kernel
int launch_md_pair_f64cells(const MDState& m, const CellsF64& c, const MDStepArgs& a, cudaStream_t s, cudaError_t* st);
int launch_md_pair_f32cells(const MDState& m, const CellsF32& c, const MDStepArgs& a, cudaStream_t s, cudaError_t* st);
int md_pair_max_coresident_blocks(const MDState& m, int f32cells);
int md_pair_threads(int tile);  // threads per CTA of the pair kernel
// reduce observables: out[0..2] sum m v, out[3] sum m v^2 (all), out[4] N, out[5] M,
// out[6] sum v^2 over fluid, out[7] N fluid
int launch_observables_f64(const FluidF64& f, const MDState& m, double bead_mass, double* out, cudaStream_t s);
// counting sort of the fluid by cell; `tmp` has the same shape as `f`
int launch_sort_f64(FluidF64& f, FluidF64& tmp, const Box& box, uint32_t* count, uint32_t* start,
                    uint32_t* rank, uint32_t* blocksums, cudaStream_t s);

int launch_cell_params_f32(const CellsF32& c, const StepArgs& a, cudaStream_t s);
// caller arrays (float64, N x 3, staged in device memory) <-> fluid layout
int launch_check_fluid(long n, const double* pos, const double* vel, unsigned* bad, cudaStream_t s);
int launch_load_fluid_f64(long n, const double* pos, const double* vel, const Box& box, const FluidF64& f,
                          cudaStream_t s);
int launch_load_fluid_f32(long n, const double* pos, const double* vel, const Box& box, const FluidF32& f,
                          cudaStream_t s);
int launch_store_fluid_f64(const FluidF64& f, double* pos, double* vel, unsigned* bad, cudaStream_t s);
int launch_store_fluid_f32(const FluidF32& f, double* pos, double* vel, unsigned* bad, cudaStream_t s);
// observables from the binned cell sums (float64 path; valid while the sums
// are those of the last binning): out[10], part[7 * kObsBlocks], counter zeroed once
constexpr int kObsBlocks = 512;
int launch_observables_cells_f64(const CellsF64& c, const MDState& m, double bead_mass, const double* diss,
                                 const unsigned* err, double* part, unsigned* counter, double* out, cudaStream_t s);
int launch_fluid_step_f32(const FluidF32& f, const CellsF32& c, const StepArgs& a, cudaStream_t s, int per_sm = 4);
int launch_bin_fluid_f32(const FluidF32& f, const CellsF32& c, const StepArgs& a, cudaStream_t s);
int launch_bead_collide_f32(const MDState& m, const CellsF32& c, const StepArgs& a, cudaStream_t s);
int launch_bin_beads_f32(const MDState& m, const CellsF32& c, const StepArgs& a, cudaStream_t s);
int launch_md_f32cells(const MDState& m, const CellsF32& c, const MDStepArgs& a, cudaStream_t s, cudaError_t* st);
int launch_md_cluster_f64cells(const MDState& m, const CellsF64& c, const MDStepArgs& a, cudaStream_t s,
                               cudaError_t* st);
int launch_md_cluster_f32cells(const MDState& m, const CellsF32& c, const MDStepArgs& a, cudaStream_t s,
                               cudaError_t* st);
int launch_observables_f32(const FluidF32& f, const MDState& m, double bead_mass, double* out, cudaStream_t s);
int launch_sort_f32(FluidF32& f, FluidF32& tmp, const Box& box, uint32_t* count, uint32_t* start,
                    uint32_t* rank, uint32_t* blocksums, cudaStream_t s);
// the generator's Gamma variates (cells of nc particles) and float64 rotation
// axes of cells 0 .. n-1 in step `step` (either output may be null)
int launch_collision_draws(int nc, uint64_t seed, uint64_t step, long n, double* gamma, double* axis, unsigned* err,
                           cudaStream_t s);
// Bead-first ordering of a step (the MD launch starts before the cell maps of
// the fluid): the collision maps of the cells that hold moving beads, each
// made once (claim[cid] takes this step's tag), ahead of the cell-map kernel
// (StepArgs::premapped); and after the MD launch the beads' deferred binning
// (MDStepArgs::deferred) added into the cell sums.
int launch_bead_maps_f64(const MDState& m, const CellsF64& c, const StepArgs& a, uint32_t* claim, uint32_t tag,
                         cudaStream_t s);
int launch_bead_maps_f32(const MDState& m, const CellsF32& c, const StepArgs& a, uint32_t* claim, uint32_t tag,
                         cudaStream_t s);
int launch_bead_add_f64(const MDState& m, const CellsF64& c, const uint32_t* bcell, const void* bsum, cudaStream_t s);
int launch_bead_add_f32(const MDState& m, const CellsF32& c, const uint32_t* bcell, const void* bsum, cudaStream_t s);
// rigid spheres after a step: force sums, motion, impulses cleared (one CTA)
int launch_spheres_update(RigidSphereDev* sph, int n, double* acc, double* fsum, double h, const Box& box,
                          cudaStream_t s);

}  // namespace mpcd
