// Host-side planning of the MD device layout: which slot every bead owns,
// the springs in CSR by slot, tile halos, cilium records.  Shared by the
// single-box engine (engine.cu) and the replica batch (batch.cu).
#pragma once
#include <string>
#include <vector>

#include "../../include/mpcd_gpu.h"
#include "engine_internal.h"

namespace mpcd {

// The bead set of one box as the setters received it (mpcd_set_beads,
// mpcd_set_springs, mpcd_set_cilia).
struct MDInput {
  long nb = 0;
  const double* bpos = nullptr;  // [nb][3]
  const double* bvel = nullptr;  // [nb][3]
  const int* bmoves = nullptr;   // [nb] 1 integrated, 0 fixed
  long nsp = 0;
  const int *sp_t = nullptr, *sp_o = nullptr, *sp_k = nullptr, *sp_r = nullptr;
  const double *sp_rest = nullptr, *sp_kk = nullptr;
  int ncil = 0;
  const mpcd_cilium* cil = nullptr;
  long nbond = 0;
  const double *newlen = nullptr, *oldlen = nullptr;
  int split = 0;  // 1: float spring arithmetic on hi/lo position pairs
  int df = 0;     // 1: double-float arithmetic (md_df.cu; grid layout, split 0)
  int pair = 0;   // with df 1: the pair kernel (md_pair.cu) on the grid layout, 1 float64, 2 double-float
};

// A fixed cluster layout (lanes per slot, slots per tile), or {0, 0} to let
// the planner search (cluster first when split, else the grid layout).
struct MDForce {
  int lanes = 0;
  int tile = 0;
};

// Host arrays of an MDState (engine_internal.h), indices local to the box.
struct MDPlan {
  int tile = 0, ntiles = 0, nslots = 0, hmax = 0;
  int split = 0, df = 0, cluster = 0, cl_nsp_max = 0, cl_nbond_max = 0, cl_lanes = 2, cl_nbuf = 2;
  std::vector<double> X, Y, Z, VX, VY, VZ;
  std::vector<int> mv, prim, nhelp, thelp, tile_react;
  std::vector<int> start, so, sl, sk, sr;
  std::vector<double> srest, sm2k;
  std::vector<int> halo, hstart;
  std::vector<CiliumDev> cd;
  std::vector<double> mid, ts, newlen, oldlen, diag;
  std::vector<int> tcil;
  std::vector<int> slot_of;  // bead -> primary slot
  // double-float grid kernel (md_df.cu)
  std::vector<int> df_split, df_b0, df_nb;
  std::vector<uint32_t> df_code;
  std::vector<int4> df_runs;       // halo runs {first slot, staged rank, length, 0}
  std::vector<int> df_run_start;  // ntiles + 1
  std::vector<int2> df_single;     // other halo entries {slot, staged rank}
  std::vector<int> df_single_start;
  int df_nsp_max = 0, df_nb_max = 0, df_nrun_max = 0, df_nsingle_max = 0;
  // pair kernel (md_pair.cu): per tile its force entries (a spring and its
  // exact reverse inside the tile form one entry), the entries reaching only
  // the tile's own beads first, those reaching a hub last; per entry the
  // incidence slots its force (and, for its second bead, the negated force)
  // is written to: a bead's incidences are its springs in its spring order,
  // so that its force is the sum of a contiguous range; per tile the beads
  // with long lists (summed by warps)
  int pair = 0;
  std::vector<int> pr_start, pr_local_end;  // ntiles + 1, ntiles (global entry offsets)
  std::vector<int> pr_hub_begin;            // ntiles: the first entry reaching a hub
  std::vector<uint2> pr_code;  // {a | b << 16, kind | both << 2 | react << 3 | bond << 4}
  std::vector<double> pr_rest, pr_m2k;
  std::vector<int> pi_start;                // nslots + 1
  std::vector<uint32_t> pr_pos;  // per entry: its first bead's incidence | its second's << 16 (0xffff: none)
  std::vector<int> pl_start, pl_list;       // ntiles + 1; local slot of each long bead
  std::vector<int> pl_base;                 // each long bead's first incidence slot
  std::vector<int> pr_nslot;                // ntiles: incidence slot words of the tile
  int pr_nent_max = 0, pr_ninc_max = 0, pr_nlong_max = 0;  // pr_ninc_max: most slot words of a tile
  // hubs of the pair kernel (engine_internal.h, HubRef)
  std::vector<int> hub_slot, hub_pbase;  // nhub, nhub + 1
  std::vector<int> th_start;             // ntiles + 1
  std::vector<HubRef> th;
  std::vector<int> tr_list;
  long nsp_kept() const { return (long)so.size(); }
};

// Plans the layout.  Returns an empty string on success, else the reason.
// `grid_f32cells` selects the co-resident limit checked for the grid layout.
// `min_tile`: the narrowest grid-layout tile to consider (0: as narrow as the
// widest cilium allows); a grid that is not co-resident is re-planned wider.
std::string plan_md(const MDInput& in, const MDForce& force, bool allow_cluster, bool no_react, int grid_f32cells,
                    MDPlan& out, int min_tile = 0);

}  // namespace mpcd
