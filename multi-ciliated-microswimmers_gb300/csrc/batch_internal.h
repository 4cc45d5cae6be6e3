// Device-side structures of the replica batch (batch.cu, batch_kernels.cu,
// md_cluster.cu): many independent boxes, each a full MPCD + swimmer system in
// split precision, advanced together.
//
// Memory: one device arena per batch.  Every replica owns
//   - a page-aligned range of fluid particles (pages of kPartPage particles),
//   - a page-aligned range of cells (pages of kCellPage cells),
//   - a range of MD tiles (plus one spare tile, see batch.cu), springs, halo
//     entries, cilia and bond-table entries, all indexed globally.
// Page tables map each page to its replica (-1 = free), so the kernels walk
// the pages and take a page's replica parameters once per page.
#pragma once
#include <cstdint>

#include "engine_internal.h"

namespace mpcd {

constexpr int kPartPage = 4096;  // fluid particles per page
constexpr int kCellPage = 1024;  // cells per page
constexpr int kMaxClusterTiles = 16;

// Per replica slot, fixed while the replica is resident.
struct BatchRep {
  int resident;        // 1 while the slot holds a replica
  int L[3];
  int walls;
  int nsub;            // MD substeps per MPC step
  long cell0, ncell;   // cell range
  long p0, n;          // fluid particle range
  int md_tile0, md_ntiles;  // MD tiles (md_ntiles = 0: no beads)
  uint64_t seed;
  double h, ststep, bead_mass, gravity, omega;
};

// Per replica, rewritten by the prologue kernel at the start of every step.
struct BatchStep {
  int active;          // takes part in this step
  uint64_t step;       // generator counter of this collision
  float fta_cur[3], fta_next[3];
  float fh, fgkick, fbead_mass;
  MDStepArgs md;       // times, refresh schedule, shifts, box (err points at the replica's word)
};

// Per replica, persistent: advanced by the prologue, read back by the host.
struct BatchState {
  uint64_t steps;          // collisions done
  long long steps_left;    // steps still to run
  double a[3];             // current grid shift
  double globalt;
  double diss;             // dissipated energy since the last reset
  unsigned err;            // kErr* bits
  unsigned pad;
};

// The arena's cell arrays (global cell index).
struct BatchCells {
  float4* sum;
  uint32_t* cnt;
  float4* par;
};

// The arena's fluid arrays (global particle index); pos/vel as FluidF32.
struct BatchFluid {
  uint32_t* id;
  float4* pos;
  float4* vel;
};

struct BatchTables {
  const BatchRep* rep;
  BatchStep* step;
  BatchState* state;
  const int* part_page_rep;  // [npart_pages]
  const int* cell_page_rep;  // [ncell_pages]
  long npart_pages, ncell_pages;
  int nrep;                  // replica slots
  // values that replace the generator for replica inj_rep in this step (as
  // mpcd_inject for one engine); inj_rep = -1: none.  Device arrays indexed by
  // the replica's own cells.
  int inj_rep = -1;
  const double* inj_shift = nullptr;  // [3]
  const double* inj_gamma = nullptr;  // [ncell]
  const double* inj_axis = nullptr;   // [ncell][3]
};

// ------------------------------------------------------------ launchers ---
int launch_batch_prologue(const BatchTables& t, cudaStream_t s);
int launch_batch_cell_params(const BatchTables& t, BatchCells c, int threads, int blocks, cudaStream_t s);
int launch_batch_fluid_step(const BatchTables& t, BatchFluid f, BatchCells c, int threads, int blocks,
                            cudaStream_t s);
// bins the fluid of pages [page0, page1) with each replica's current shift
int launch_batch_bin_fluid(const BatchTables& t, BatchFluid f, BatchCells c, long page0, long page1, cudaStream_t s);
// bins the MD beads of tiles [tile0, tile1) with each replica's current shift
int launch_batch_bin_beads(const BatchTables& t, const MDState& m, const int* tile_rep, BatchCells c, int tile0,
                           int tile1, cudaStream_t s);
// counting sort of every resident replica's fluid within its own range
int launch_batch_sort(const BatchTables& t, BatchFluid src, BatchFluid dst, uint32_t* count, uint32_t* start,
                      uint32_t* rank, uint32_t* blocksums, long ncell_total, cudaStream_t s);
// per replica: out[8 * r + k] as launch_observables_f32's eight sums
int launch_batch_observables(const BatchTables& t, BatchFluid f, const MDState& m, const int* tile_rep, int ntiles,
                             double* out, cudaStream_t s);
// MD of the replicas listed in `reps` (all with `ctiles` tiles), one cluster each
int launch_md_cluster_batch(const MDState& m, const BatchTables& t, BatchCells c, const int* reps, int nreps,
                            int ctiles, int hmax, int nsp_max, int nbond_max, int nbuf, cudaStream_t s,
                            cudaError_t* st);
// shared memory of one CTA; nbuf position buffers (2, or 1 with a second cluster barrier per substep)
size_t md_cluster_batch_smem(int tile, int hmax, int nsp_max, int nbond_max, int nbuf);
int md_cluster_batch_feasible(int lanes, int tile, int ctiles, size_t smem);

// shared with fluid_kernels.cu: exclusive scan of `count` into `start`
int scan_counts_ext(const uint32_t* count, long ncell, uint32_t* start, uint32_t* blocksums, cudaStream_t s);

}  // namespace mpcd
