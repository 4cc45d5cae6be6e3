// MD substeps of one MPC step in IEEE float64, each spring pair evaluated once.
//
// Same integrator and forces as md_kernels.cu (velocity Verlet of
// src/libcilia/mdobject.cpp:36-72 inside the loop of src/simulation.cpp:217-265;
// springs of src/cilia.cpp:127-239, src/sphere.cpp:87-119, src/clami.cpp:188-198)
// on the cooperative-grid tile layout of md_df.cu with one slot per bead.
//
// GB300 issues float64 at about two fused multiply-adds per clock per SM, so
// a float64 MD step is bound by how many float64 instructions the busiest SM
// issues.  The reference makes every cilium and sphere spring twice, once from
// each end (MDObject::spring is one-sided); the two forces are exact negations
// of each other.  Here a tile's springs become force entries: a spring and its
// reverse inside the tile are one entry, evaluated once by one thread (all
// threads of the CTA take entries in turn, so no lane idles on a short list),
// and every bead sums the entries of its springs, negating where it is the
// entry's second bead, in its own spring order (a fixed order: the result
// does not depend on timing).  A bead with a long list (a sphere's centre) is
// summed by warps: lane-strided, then a xor tree.
//
// Positions are exchanged between tiles through two global buffers of four
// float64 per slot after a bounded grid barrier, the halo arriving by bulk
// asynchronous copies (TMA) and cp.async while the entries between the tile's
// own beads are evaluated.  The cilia's rest lengths: the beat's target of
// every bond is fixed during one MPC step's substeps and computed once per
// launch; the bending-rate limit runs at every refresh (every 0.01 time units).
#include <cstdlib>

#include "../../include/mpcd_gpu.h"
#include "md_common.cuh"
#include "tma.cuh"

namespace mpcd {

namespace {

constexpr uint32_t kPairHaloWait = 1u << 22;  // polls of the halo's mbarrier before giving up

__device__ __forceinline__ void cp_async16_p(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all_p() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// a staged or published position: x, y, z and one unused word (32 bytes, so
// that runs of slots copy as whole 16-byte units)
struct __align__(16) Pos4 {
  double x, y, z, w;
};

// v, negated when bit 0 of w is set: the sign bit flipped by an integer
// operation, so that a bead's sum costs one float64 add per entry
__device__ __forceinline__ double flip_sign(double v, uint32_t w) {
  return __hiloint2double(__double2hiint(v) ^ (int)((w & 1u) << 31), __double2loint(v));
}

// 1 / sqrt(d2) for a positive normal d2: the float reciprocal square root
// (relative error about 2^-23) refined by one cubic step of the Householder
// iteration for f(y) = y^-2 - d2: with r = 1 - d2 y^2, y' = y + y r (1/2 + 3/8 r),
// whose error is of order r^3 (about 2^-69), below float64 rounding; five
// float64 operations
__device__ __forceinline__ double rsqrt_f64(double d2) {
  const double y = (double)rsqrtf((float)d2);
  const double r = fma(-d2 * y, y, 1.0);
  return fma(y * r, fma(0.375, r, 0.5), y);
}

struct StagePair {
  const Pos4* p;
  __device__ double dist(int i, int j) const {
    const double dx = p[i].x - p[j].x, dy = p[i].y - p[j].y, dz = p[i].z - p[j].z;
    return sqrt(dx * dx + dy * dy + dz * dz);
  }
};

// shared-memory layout of one tile
struct PairSmem {
  size_t st, bar, flag, runs, single, code, rest, m2k, fx, fy, fz, inc, incs, lng, nl, ol, dg, tg, bd, fs, total;
  __host__ __device__ PairSmem(int T, int hmax, int nent, int ninc, int nlong, int nb, int nrun, int nsingle) {
    size_t o = 0;
    auto take = [&](size_t bytes, size_t align) {
      o = (o + align - 1) / align * align;
      const size_t r = o;
      o += bytes;
      return r;
    };
    st = take(sizeof(Pos4) * (size_t)(T + hmax), 16);
    bar = take(8, 8);
    flag = take(4, 4);
    runs = take(16 * (size_t)nrun, 16);
    single = take(8 * (size_t)nsingle, 8);
    code = take(8 * (size_t)nent, 8);
    rest = take(8 * (size_t)nent, 8);
    m2k = take(8 * (size_t)nent, 8);
    fx = take(8 * (size_t)nent, 8);
    fy = take(8 * (size_t)nent, 8);
    fz = take(8 * (size_t)nent, 8);
    nl = take(8 * (size_t)nb, 8);
    ol = take(8 * (size_t)nb, 8);
    dg = take(8 * (size_t)nb, 8);
    tg = take(8 * (size_t)nb, 8);
    bd = take(8 * (size_t)nb, 8);
    fs = take(24 * (size_t)T, 8);
    inc = take(4 * (size_t)ninc, 4);
    incs = take(4 * (size_t)(T + 1), 4);
    lng = take(4 * (size_t)nlong, 4);
    total = o;
  }
};

__host__ __device__ inline PairSmem pair_smem(const MDState& m) {
  return PairSmem(m.tile, m.hmax, m.pr_nent_max, m.pr_ninc_max, m.pr_nlong_max, m.df_nb_max, m.df_nrun_max,
                  m.df_nsingle_max);
}

template <typename Bin>
__device__ void md_pair_body(const MDState& m, const MDStepArgs& a, Bin bin) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int T = m.tile;
  const PairSmem L = pair_smem(m);
  Pos4* st = reinterpret_cast<Pos4*>(smem + L.st);
  uint64_t* hbar = reinterpret_cast<uint64_t*>(smem + L.bar);  // halo copies' completion
  int* hflag = reinterpret_cast<int*>(smem + L.flag);           // 1: the plan is consistent
  int4* s_runs = reinterpret_cast<int4*>(smem + L.runs);
  int2* s_single = reinterpret_cast<int2*>(smem + L.single);
  uint2* s_code = reinterpret_cast<uint2*>(smem + L.code);
  double* s_rest = reinterpret_cast<double*>(smem + L.rest);
  double* s_m2k = reinterpret_cast<double*>(smem + L.m2k);
  double* s_fx = reinterpret_cast<double*>(smem + L.fx);  // per entry: force on its first bead
  double* s_fy = reinterpret_cast<double*>(smem + L.fy);
  double* s_fz = reinterpret_cast<double*>(smem + L.fz);
  double* s_nl = reinterpret_cast<double*>(smem + L.nl);  // bonds: current rest length
  double* s_ol = reinterpret_cast<double*>(smem + L.ol);  // previous rest length
  double* s_dg = reinterpret_cast<double*>(smem + L.dg);  // diagonal rest length
  double* s_tg = reinterpret_cast<double*>(smem + L.tg);  // the beat's target for this step
  double* s_bd = reinterpret_cast<double*>(smem + L.bd);  // bending-rate limit
  double* s_fs = reinterpret_cast<double*>(smem + L.fs);  // per axis and bead: its summed force
  uint32_t* s_inc = reinterpret_cast<uint32_t*>(smem + L.inc);
  int* s_incs = reinterpret_cast<int*>(smem + L.incs);
  int* s_lng = reinterpret_cast<int*>(smem + L.lng);
  const StagePair sv{st};

  const int tile = blockIdx.x;
  const int base = tile * T;
  const int tid = threadIdx.x;
  const int nthr = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarps = nthr >> 5;
  // bead owners: thread tid < T owns slot base + tid
  const int oslot = base + tid;
  const int omv = tid < T ? m.moves[oslot] : -1;
  const bool oprim = omv == 0 || omv == 1, omoves = omv == 1;
  const int h0 = m.halo_start[tile], hn0 = m.halo_start[tile + 1] - h0;
  const int c0 = m.tile_cil[tile], c1 = m.tile_cil[tile + 1];
  const int b0 = m.tile_b0[tile], nb = m.tile_nb[tile];
  const int e0 = m.pr_start[tile], nent0 = m.pr_start[tile + 1] - e0, nloc0 = m.pr_local_end[tile] - e0;
  const int i0 = m.pi_start[base], ninc0 = m.pi_start[base + T] - i0;
  const int l0 = m.pl_start[tile], nlong0 = m.pl_start[tile + 1] - l0;
  const int t0h = m.th_start[tile], nth0 = m.th_start[tile + 1] - t0h;
  const double dt = a.dt;
  // hubs this tile owns or reaches, and its copy of each one's state (x, v)
  __shared__ HubRef s_href[kTileHubs];
  __shared__ double s_hst[kTileHubs][6];

  const int r0 = m.halo_run_start[tile], nrun = m.halo_run_start[tile + 1] - r0;
  const int s0 = m.halo_single_start[tile], nsingle = m.halo_single_start[tile + 1] - s0;
  for (int r = tid; r < nrun && nrun <= m.df_nrun_max; r += nthr) s_runs[r] = m.halo_run[r0 + r];
  for (int i = tid; i < nsingle && nsingle <= m.df_nsingle_max; i += nthr) s_single[i] = m.halo_single[s0 + i];
  if (tid == 0) {
    // every copy must stay inside the staged halo and the position buffers,
    // the copies must cover the halo exactly, and the tables must fit
    int ok = 1, tot = nsingle;
    for (int r = 0; r < nrun; ++r) {
      const int4 run = m.halo_run[r0 + r];
      ok &= run.z > 0 && run.y >= 0 && run.y + run.z <= m.hmax && run.x >= 0 && run.x + run.z <= m.nslots;
      tot += run.z;
    }
    for (int i = 0; i < nsingle; ++i) {
      const int2 e = m.halo_single[s0 + i];
      ok &= e.y >= 0 && e.y < m.hmax && e.x >= 0 && e.x < m.nslots;
    }
    // a hub in the halo keeps its staged place but is not copied
    int nhh = 0;
    ok &= nth0 >= 0 && nth0 <= kTileHubs;
    for (int j = 0; j < nth0 && j < kTileHubs; ++j) {
      const HubRef r = m.th[t0h + j];
      ok &= r.hub >= 0 && r.hub < m.nhub && r.idx >= 0 && r.idx < T + hn0 && r.rs >= 0 && r.rn >= 0 &&
            r.rs + r.rn <= m.ntr;
      if (ok)
        ok &= r.rank < m.hub_pbase[r.hub + 1] - m.hub_pbase[r.hub] && m.hub_slot[r.hub] >= 0 &&
              m.hub_slot[r.hub] < m.nslots;
      nhh += r.idx >= T;
      s_href[j] = r;
    }
    ok &= tot + nhh == hn0 && nrun <= m.df_nrun_max && nsingle <= m.df_nsingle_max;
    ok &= nent0 >= 0 && nent0 <= m.pr_nent_max && nloc0 >= 0 && nloc0 <= nent0 && ninc0 >= 0 &&
          ninc0 <= m.pr_ninc_max && nlong0 >= 0 && nlong0 <= m.pr_nlong_max && nb >= 0 && nb <= m.df_nb_max;
    if (!ok) atomicOr(a.err, kErrLayout);
    *hflag = ok;
    mbar_init(hbar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  // an inconsistent plan: no halo copies, no entries (and an error)
  const bool plan_ok = *hflag != 0;
  const int hn = plan_ok ? hn0 : 0;
  const int nent = plan_ok ? nent0 : 0, nloc = plan_ok ? nloc0 : 0, ninc = plan_ok ? ninc0 : 0;
  const int nlong = plan_ok ? nlong0 : 0, nbt = plan_ok ? nb : 0;
  const int nth = plan_ok ? nth0 : 0;
  bool ohub = false;  // the owned bead is a hub: integrated from partial sums, not by its thread
  for (int j = 0; j < nth; ++j) ohub = ohub || s_href[j].idx == tid;
  uint32_t long_bytes = 0;
  if (plan_ok)
    for (int r = 0; r < nrun; ++r) long_bytes += (uint32_t)sizeof(Pos4) * (uint32_t)s_runs[r].z;
  uint32_t hphase = 0;
  // tile-resident tables; entries and incidences are checked against the staged range
  for (int i = tid; i < nent; i += nthr) {
    uint2 c = __ldg(m.pr_code + e0 + i);
    const int ea = (int)(c.x & 0xffffu), eb = (int)(c.x >> 16), lref = (int)(c.y >> 4);
    const int kind = (int)(c.y & 3u);
    if (ea >= T || eb >= T + hn || (kind >= MPCD_SPRING_BOND && lref >= nbt)) {
      atomicOr(a.err, kErrLayout);
      c = make_uint2(0u, 0u);  // bead 0 against itself: no access outside the tables
    }
    s_code[i] = c;
    s_rest[i] = __ldg(m.pr_rest + e0 + i);
    s_m2k[i] = __ldg(m.pr_m2k + e0 + i);
  }
  for (int i = tid; i < ninc; i += nthr) {
    uint32_t w = __ldg(m.pi_list + i0 + i);
    if ((int)(w >> 1) >= nent) {
      atomicOr(a.err, kErrLayout);
      w = 0u;
    }
    s_inc[i] = w;
  }
  for (int i = tid; i <= T; i += nthr) s_incs[i] = plan_ok ? min(max(m.pi_start[base + i] - i0, 0), ninc) : 0;
  for (int i = tid; i < nlong; i += nthr) s_lng[i] = min(max(m.pl_list[l0 + i], 0), T - 1);
  for (int i = tid; i < nbt; i += nthr) {
    s_nl[i] = m.newlen[b0 + i];
    s_ol[i] = m.oldlen[b0 + i];
    s_dg[i] = m.diag[b0 + i];
  }
  // the beat's rest length of every refreshed bond for this step, and the bending limit
  {
    int off = 0;
    for (int c = c0; c < c1; ++c) {
      const CiliumDev cl = m.cil[c];
      const int nbnd = cl.len - cl.num_anker;
      const int w = tid - off;
      if (w >= 0 && w < nbnd) {
        const int i = cl.num_anker - 1 + w;
        const int k = cl.bond_base + i - b0;
        if (k >= 0 && k < nbt) {
          s_tg[k] = cilium_target(cl, i, m.midpnt[c]);
          s_bd[k] = cl.bending;
        }
      }
      off += nbnd;
    }
  }
  double x = 0, y = 0, z = 0, vx = 0, vy = 0, vz = 0, fx = 0, fy = 0, fz = 0;
  double ke_coll = 0.0;
  if (oprim) {
    x = m.x[0][oslot];
    y = m.y[0][oslot];
    z = m.z[0][oslot];
    vx = m.vx[oslot];
    vy = m.vy[oslot];
    vz = m.vz[oslot];
    if (a.collide && omoves) ke_coll = bin.collide(x, y, z, vx, vy, vz);  // the beads' collision, folded in
  }
  if (tid < nth) {
    // a hub's state at the start of the step, after the beads' collision as
    // its owner applies it (the same arithmetic on the same values)
    const HubRef r = s_href[tid];
    const int hs = m.hub_slot[r.hub];
    double X = m.x[0][hs], Y = m.y[0][hs], Z = m.z[0][hs];
    double VX = m.vx[hs], VY = m.vy[hs], VZ = m.vz[hs];
    if (a.collide && m.moves[hs] == 1) (void)bin.collide(X, Y, Z, VX, VY, VZ);
    s_hst[tid][0] = X;
    s_hst[tid][1] = Y;
    s_hst[tid][2] = Z;
    s_hst[tid][3] = VX;
    s_hst[tid][4] = VY;
    s_hst[tid][5] = VZ;
    Pos4 p;
    p.x = X;
    p.y = Y;
    p.z = Z;
    p.w = 0.0;
    st[r.idx] = p;
  }
  if (a.collide) {  // the dissipated-energy bookkeeping of the collided beads
    const double tot = block_sum_f64(ke_coll);
    if (tid == 0 && tot != 0.0) atomicAdd(a.diss, -tot);
  }
  Pos4* q[2] = {reinterpret_cast<Pos4*>(m.q[0]), reinterpret_cast<Pos4*>(m.q[1])};
  const unsigned nblocks = gridDim.x;
  unsigned barriers = 0;
  int eval = 0;
  bool refreshed = false;

  // own beads into shared memory and the global buffer b
  auto publish = [&](int b) {
    if (oprim && !ohub) {
      Pos4 p;
      p.x = x;
      p.y = y;
      p.z = z;
      p.w = 0.0;
      st[tid] = p;
      q[b][oslot] = p;
    }
  };
  // entry i: F = -2k (1 - b / |d|) d, d = x_a - x_b (MDObject::spring, src/libcilia/mdobject.cpp:8-29)
  auto entry = [&](int i) {
    const uint2 c = s_code[i];
    const int ea = (int)(c.x & 0xffffu), eb = (int)(c.x >> 16);
    const int kind = (int)(c.y & 3u), lref = (int)(c.y >> 4);
    const double rl = kind <= MPCD_SPRING_GUARDED ? s_rest[i] : (kind == MPCD_SPRING_BOND ? s_nl[lref] : s_dg[lref]);
    const Pos4 pa = st[ea], pb = st[eb];
    const double dx = pa.x - pb.x, dy = pa.y - pb.y, dz = pa.z - pb.z;
    const double d2 = dx * dx + dy * dy + dz * dz;
    double gx = 0.0, gy = 0.0, gz = 0.0;
    if (!(kind == MPCD_SPRING_GUARDED && d2 == 0.0)) {  // vector-form spring: no force at zero distance
      const double fac = s_m2k[i] * (1.0 - rl * rsqrt_f64(d2));
      gx = dx * fac;
      gy = dy * fac;
      gz = dz * fac;
    }
    s_fx[i] = gx;
    s_fy[i] = gy;
    s_fz[i] = gz;
  };
  // hub j's force from evaluation e: the published partial sums of its
  // contributors (four float64 each) in their order, lane-strided and then by
  // a xor tree (every lane, and every tile, gets the same number); called by
  // a whole warp
  auto hub_force = [&](int j, int e, double& sx, double& sy, double& sz) {
    const HubRef r = s_href[j];
    const int p0 = m.hub_pbase[r.hub], nc = m.hub_pbase[r.hub + 1] - p0;
    const double* P = m.hubpart + ((size_t)(e & 1) * m.hub_ncon + p0) * 4;
    sx = sy = sz = 0.0;
    for (int c = lane; c < nc; c += 32) {
      sx += __ldcg(P + 4 * c);
      sy += __ldcg(P + 4 * c + 1);
      sz += __ldcg(P + 4 * c + 2);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sx += __shfl_xor_sync(0xffffffffu, sx, o);
      sy += __shfl_xor_sync(0xffffffffu, sy, o);
      sz += __shfl_xor_sync(0xffffffffu, sz, o);
    }
  };
  // before evaluation e >= 1 (after its grid barrier): the last warps, one
  // per hub, advance the tile's copy of hub j with the force of evaluation
  // e - 1, as the Verlet steps of the owned beads, and stage its position,
  // while the other warps evaluate the entries between the tile's own beads
  auto hub_update = [&](int e) {
    const int j = nwarps - 1 - warp;
    if (j < 0 || j >= nth) return;
    const HubRef r = s_href[j];
    double sx, sy, sz;
    hub_force(j, e - 1, sx, sy, sz);
    if (lane == 0) {
      double* hs = s_hst[j];
      if (m.moves[m.hub_slot[r.hub]] == 1) {
        const double c = e == 1 ? dt / 2.0 : dt;
        hs[3] = fma(sx, c, hs[3]);
        hs[4] = fma(sy, c, hs[4]);
        hs[5] = fma(sz, c, hs[5]);
        hs[0] = fma(hs[3], dt, hs[0]);
        hs[1] = fma(hs[4], dt, hs[1]);
        hs[2] = fma(hs[5], dt, hs[2]);
      }
      Pos4 p;
      p.x = hs[0];
      p.y = hs[1];
      p.z = hs[2];
      p.w = 0.0;
      st[r.idx] = p;
    }
  };
  // forces on the owned beads; buffer b holds the other tiles' beads
  auto evaluate = [&](int b) {
    const int ev = eval;
    if (hn > 0) {
      // the other tiles wrote the buffer through the generic proxy; order
      // those writes (acquired at the barrier) before this thread's bulk reads
      if (tid < nrun) asm volatile("fence.proxy.async.global;" ::: "memory");
      for (int r = tid; r < nrun; r += nthr) {
        const int4 run = s_runs[r];
        bulk_load(st + T + run.y, q[b] + run.x, (uint32_t)sizeof(Pos4) * (uint32_t)run.z, hbar);
      }
      for (int i = tid; i < nsingle; i += nthr) {
        const int2 e = s_single[i];
        cp_async16_p(reinterpret_cast<double*>(st + T + e.y), reinterpret_cast<const double*>(q[b] + e.x));
        cp_async16_p(reinterpret_cast<double*>(st + T + e.y) + 2, reinterpret_cast<const double*>(q[b] + e.x) + 2);
      }
    }
    const bool hubs_due = ev >= 1 && nth > 0;
    if (c1 > c0 && refresh_due(a, eval)) {
      // Cilia::length (src/cilia.cpp:79-121) for every refreshed bond
      refreshed = true;
      int off = 0;
      for (int c = c0; c < c1; ++c) {
        const CiliumDev cl = m.cil[c];
        const int nbnd = cl.len - cl.num_anker;
        const int w = tid - off;
        if (w >= 0 && w < nbnd && cl.bond_base + cl.num_anker - 1 + w - b0 < nbt) {
          const int i = cl.num_anker - 1 + w;
          const int k = cl.bond_base + i - b0;
          const int lb = cl.slot0 - base;
          const double l = cilium_limit(s_tg[k], s_bd[k], s_ol[k], sv.dist(lb + cl.stride * i, lb + cl.stride * (i + 1)));
          s_nl[k] = l;
          s_ol[k] = l;
          s_dg[k] = sqrt(0.5 * 0.5 + 0.5 * l);
        }
        off += nbnd;
      }
      __syncthreads();
    }
    ++eval;
    {
      // the entries between the tile's own beads, beside the hubs' update
      const int ethr = hubs_due ? nthr - 32 * nth : nthr;
      if (tid < ethr)
        for (int i = tid; i < nloc; i += ethr) entry(i);
      if (hubs_due) hub_update(ev);
    }
    if (hn > 0 || hubs_due) {
      if (long_bytes) {
        if (!mbar_wait(hbar, hphase & 1u, kPairHaloWait)) atomicOr(a.err, kErrBarrier);
        ++hphase;
      }
      cp_async_wait_all_p();
      __syncthreads();
    }
    for (int i = nloc + tid; i < nent; i += nthr) entry(i);
    // the halo region is refilled by the async proxy next substep
    fence_proxy_async_smem();
    __syncthreads();
    // every bead sums its entries in its spring order: a thread per bead and
    // axis, a warp per bead and axis for long lists
    for (int w = tid; w < 3 * T; w += nthr) {
      const int bd = w / 3, ax = w - 3 * bd;
      const int k0 = s_incs[bd], k1 = s_incs[bd + 1];
      if (k1 - k0 > kPairLong) continue;
      const double* F = ax == 0 ? s_fx : (ax == 1 ? s_fy : s_fz);
      // two chains (alternate entries), then their sum: a fixed order
      double s = 0.0, t = 0.0;
      int k = k0;
      for (; k + 1 < k1; k += 2) {
        const uint32_t e = s_inc[k], f = s_inc[k + 1];
        s += flip_sign(F[e >> 1], e);
        t += flip_sign(F[f >> 1], f);
      }
      if (k < k1) s += flip_sign(F[s_inc[k] >> 1], s_inc[k]);
      s_fs[ax * T + bd] = s + t;
    }
    for (int w = warp; w < 3 * nlong; w += nwarps) {
      const int bd = s_lng[w / 3], ax = w % 3;
      const int k0 = s_incs[bd], k1 = s_incs[bd + 1];
      const double* F = ax == 0 ? s_fx : (ax == 1 ? s_fy : s_fz);
      double s = 0.0;
      for (int k = k0 + lane; k < k1; k += 32) {
        const uint32_t e = s_inc[k];
        s += flip_sign(F[e >> 1], e);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) s_fs[ax * T + bd] = s;
    }
    // the reactions this tile owes each hub: the negated sum of its entries
    // to the hub, in entry order (lane-strided, xor tree), published for the
    // hub's copies after the next grid barrier
    // (by the last warps, beside the sums of the first ones)
    for (int w = nwarps - 1 - warp; w < 3 * nth; w += nwarps) {
      const HubRef r = s_href[w / 3];
      const int ax = w % 3;
      if (r.rank < 0) continue;
      const double* F = ax == 0 ? s_fx : (ax == 1 ? s_fy : s_fz);
      double s = 0.0;
      for (int k = lane; k < r.rn; k += 32) {
        const int ei = __ldg(m.tr_list + r.rs + k);
        if (ei >= 0 && ei < nent) s -= F[ei];
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) m.hubpart[((size_t)(ev & 1) * m.hub_ncon + m.hub_pbase[r.hub] + r.rank) * 4 + ax] = s;
    }
    __syncthreads();
    if (oprim) {
      fx = s_fs[tid];
      fy = s_fs[T + tid];
      fz = s_fs[2 * T + tid];
    }
  };
  // the grid barrier before every evaluation; the halo's mbarrier is armed
  // with the next copies' bytes before any of them can be issued
  auto barrier = [&]() {
    if (tid == 0 && long_bytes) mbar_arrive_expect_tx(hbar, long_bytes);
    return grid_sync(m.bar, ++barriers * nblocks, a.err);
  };

  // md_loop_start: forces at t0, v += F dt/2, x += v dt
  const bool kicks = omoves && !ohub;  // a hub moves by its copies (hub_update)
  publish(0);
  if (!barrier()) return;
  evaluate(0);
  int cur = 0;
  if (kicks) {
    vx = fma(fx, dt / 2.0, vx);
    vy = fma(fy, dt / 2.0, vy);
    vz = fma(fz, dt / 2.0, vz);
    x = fma(vx, dt, x);
    y = fma(vy, dt, y);
    z = fma(vz, dt, z);
  }
  publish(cur ^ 1);
  if (!barrier()) return;
  cur ^= 1;
  evaluate(cur);
  // md_loop: v += F dt, x += v dt, forces
  for (int k = 1; k < a.n; ++k) {
    if (kicks) {
      vx = fma(fx, dt, vx);
      vy = fma(fy, dt, vy);
      vz = fma(fz, dt, vz);
      x = fma(vx, dt, x);
      y = fma(vy, dt, y);
      z = fma(vz, dt, z);
    }
    publish(cur ^ 1);
    if (!barrier()) return;
    cur ^= 1;
    evaluate(cur);
  }
  // md_loop_stop: v += F dt/2, then bin with the next shift
  if (kicks) {
    vx = fma(fx, dt / 2.0, vx);
    vy = fma(fy, dt / 2.0, vy);
    vz = fma(fz, dt / 2.0, vz);
  }
  if (oprim && !ohub) {
    m.x[0][oslot] = x;
    m.y[0][oslot] = y;
    m.z[0][oslot] = z;
    m.vx[oslot] = vx;
    m.vy[oslot] = vy;
    m.vz[oslot] = vz;
    if (omoves) {
      if (a.deferred)
        bin.defer(oslot, x, y, z, vx, vy, vz);
      else
        bin(x, y, z, vx, vy, vz);
    }
  }
  if (m.nhub > 0) {
    // the last evaluation's partial sums reach the hubs after one more grid
    // barrier; each owner finishes its hub: v += F dt/2, state out, binning
    if (!grid_sync(m.bar, ++barriers * nblocks, a.err)) return;
    if (warp < nth && s_href[warp].idx < T) {
      const HubRef r = s_href[warp];
      double sx, sy, sz;
      hub_force(warp, eval - 1, sx, sy, sz);
      if (lane == 0) {
        const int hs = m.hub_slot[r.hub];
        double* h = s_hst[warp];
        const bool mv = m.moves[hs] == 1;
        if (mv) {
          h[3] = fma(sx, dt / 2.0, h[3]);
          h[4] = fma(sy, dt / 2.0, h[4]);
          h[5] = fma(sz, dt / 2.0, h[5]);
        }
        m.x[0][hs] = h[0];
        m.y[0][hs] = h[1];
        m.z[0][hs] = h[2];
        m.vx[hs] = h[3];
        m.vy[hs] = h[4];
        m.vz[hs] = h[5];
        if (mv) {
          if (a.deferred)
            bin.defer(hs, h[0], h[1], h[2], h[3], h[4], h[5]);
          else
            bin(h[0], h[1], h[2], h[3], h[4], h[5]);
        }
      }
    }
  }
  // refreshed bonds back to the global tables
  if (refreshed) {
    int off = 0;
    for (int c = c0; c < c1; ++c) {
      const CiliumDev cl = m.cil[c];
      const int nbnd = cl.len - cl.num_anker;
      const int w = tid - off;
      if (w >= 0 && w < nbnd) {
        const int k = cl.bond_base + cl.num_anker - 1 + w;
        if (k - b0 >= 0 && k - b0 < nbt) {
          m.newlen[k] = s_nl[k - b0];
          m.oldlen[k] = s_ol[k - b0];
          m.diag[k] = s_dg[k - b0];
        }
      }
      off += nbnd;
    }
  }
  // switch_logic for the cilia of this tile (the staged positions are the final ones)
  for (int c = c0 + tid; c < c1; c += nthr) cilium_switch(m, a, c, a.t_end, base, sv);
  __syncthreads();
  if (tid == 0) mbar_inval(hbar);
}

template <typename Bin>
__global__ void __launch_bounds__(512) k_md_pair(MDState m, typename Bin::Cells c, MDStepArgs a) {
  md_pair_body(m, a, Bin{c, &a});
}

size_t md_pair_smem(const MDState& m) { return pair_smem(m).total; }

template <typename Bin>
int launch_pair(const MDState& m, const typename Bin::Cells& c, const MDStepArgs& a, cudaStream_t s,
                cudaError_t* st) {
  if (m.nslots == 0 || m.ntiles == 0) return 0;
  cudaMemsetAsync(m.bar.count, 0, 2 * sizeof(unsigned), s);  // count and gen are adjacent
  MDState mm = m;
  typename Bin::Cells cc = c;
  MDStepArgs aa = a;
  void* args[] = {&mm, &cc, &aa};
  const size_t smem = md_pair_smem(m);
  const void* k = (const void*)k_md_pair<Bin>;
  if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  *st = cudaLaunchCooperativeKernel(k, dim3(m.ntiles), dim3(md_pair_threads(m.tile)), args, smem, s);
  return 1;
}

}  // namespace

// enough threads for a thread per owned bead and axis in the force sums
int md_pair_threads(int tile) { return tile <= 64 ? 256 : (tile <= 128 ? 384 : 512); }

int launch_md_pair_f64cells(const MDState& m, const CellsF64& c, const MDStepArgs& a, cudaStream_t s,
                            cudaError_t* st) {
  return launch_pair<BinF64>(m, c, a, s, st);
}

int launch_md_pair_f32cells(const MDState& m, const CellsF32& c, const MDStepArgs& a, cudaStream_t s,
                            cudaError_t* st) {
  return launch_pair<BinF32>(m, c, a, s, st);
}

int md_pair_max_coresident_blocks(const MDState& m, int f32cells) {
  int dev = 0, sms = 0, per_sm = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t smem = md_pair_smem(m);
  if (smem > (size_t)optin) return 0;
  const void* k = f32cells ? (const void*)k_md_pair<BinF32> : (const void*)k_md_pair<BinF64>;
  if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, md_pair_threads(m.tile), smem);
  return per_sm * sms;
}

}  // namespace mpcd
