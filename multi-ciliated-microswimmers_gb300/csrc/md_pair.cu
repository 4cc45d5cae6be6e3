// MD substeps of one MPC step, each spring pair evaluated once: in IEEE
// float64, or in double-float arithmetic on the FP32 pipes (the arithmetic of
// md_df.cu, on this layout).
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
//
// The double-float instance keeps every bead as an integer cell plus a float
// pair offset (md_df_coord.cuh) and the velocities, forces and sums as float
// pairs; an entry's force is the double-float spring of md_df.cu, and the
// sums are compensated.  Its dependent chains run on the FP32 pipes, whose
// latency is a small fraction of the float64 pipe's on GB300.
#include <cstdlib>
#include <type_traits>

#include "../../include/mpcd_gpu.h"
#include "df32.cuh"
#include "md_common.cuh"
#include "md_df_coord.cuh"
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

struct StagePair {
  const Pos4* p;
  __device__ double dist(int i, int j) const {
    const double dx = p[i].x - p[j].x, dy = p[i].y - p[j].y, dz = p[i].z - p[j].z;
    return sqrt(dx * dx + dy * dy + dz * dz);
  }
};

// a hub's copy in one tile: float64 position and velocity, or cell + pair
// coordinates and pair velocities
struct HubF64 {
  double x[3], v[3];
};
struct HubDF {
  BeadCoord x[3];
  dfloat v[3];
};

// shared-memory layout of one tile (8-byte table and force words: a float64
// or a float pair)
struct PairSmem {
  size_t st, bar, flag, runs, single, code, rest, m2k, fx, fy, fz, pos, incs, lng, nl, ol, dg, tg, bd, fs, total;
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
    fx = take(8 * (size_t)ninc, 8);  // forces per incidence slot
    fy = take(8 * (size_t)ninc, 8);
    fz = take(8 * (size_t)ninc, 8);
    nl = take(8 * (size_t)nb, 8);
    ol = take(8 * (size_t)nb, 8);
    dg = take(8 * (size_t)nb, 8);
    tg = take(8 * (size_t)nb, 8);
    bd = take(8 * (size_t)nb, 8);
    fs = take(24 * (size_t)T, 8);
    pos = take(4 * (size_t)nent, 4);
    incs = take(4 * (size_t)(T + 1), 4);
    lng = take(8 * (size_t)nlong, 8);
    total = o;
  }
};

__host__ __device__ inline PairSmem pair_smem(const MDState& m) {
  return PairSmem(m.tile, m.hmax, m.pr_nent_max, m.pr_ninc_max, m.pr_nlong_max, m.df_nb_max, m.df_nrun_max,
                  m.df_nsingle_max);
}

template <bool kDF, typename Bin>
__device__ void md_pair_body(const MDState& m, const MDStepArgs& a, Bin bin) {
  using W = std::conditional_t<kDF, float2, double>;  // one table or force word
  extern __shared__ __align__(16) unsigned char smem[];
  const int T = m.tile;
  const PairSmem L = pair_smem(m);
  float4* st = reinterpret_cast<float4*>(smem + L.st);  // two float4 per staged bead
  Pos4* sp = reinterpret_cast<Pos4*>(st);                // the same, as float64 positions
  uint64_t* hbar = reinterpret_cast<uint64_t*>(smem + L.bar);  // halo copies' completion
  int* hflag = reinterpret_cast<int*>(smem + L.flag);           // 1: the plan is consistent
  int4* s_runs = reinterpret_cast<int4*>(smem + L.runs);
  int2* s_single = reinterpret_cast<int2*>(smem + L.single);
  uint2* s_code = reinterpret_cast<uint2*>(smem + L.code);
  W* s_rest = reinterpret_cast<W*>(smem + L.rest);
  W* s_m2k = reinterpret_cast<W*>(smem + L.m2k);
  W* s_fx = reinterpret_cast<W*>(smem + L.fx);  // per incidence slot: the force its spring puts on its bead
  W* s_fy = reinterpret_cast<W*>(smem + L.fy);
  W* s_fz = reinterpret_cast<W*>(smem + L.fz);
  W* s_nl = reinterpret_cast<W*>(smem + L.nl);  // bonds: current rest length
  W* s_ol = reinterpret_cast<W*>(smem + L.ol);  // previous rest length
  W* s_dg = reinterpret_cast<W*>(smem + L.dg);  // diagonal rest length
  W* s_tg = reinterpret_cast<W*>(smem + L.tg);  // the beat's target for this step
  W* s_bd = reinterpret_cast<W*>(smem + L.bd);  // bending-rate limit
  W* s_fs = reinterpret_cast<W*>(smem + L.fs);  // per axis and bead: its summed force
  uint32_t* s_pos = reinterpret_cast<uint32_t*>(smem + L.pos);  // per entry: its incidence slots
  int* s_incs = reinterpret_cast<int*>(smem + L.incs);
  int2* s_lng = reinterpret_cast<int2*>(smem + L.lng);  // long beads: local slot, first incidence slot
  const StagePair sv64{sp};
  const StageDF svdf{st};

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
  const int i0 = m.pi_start[base], ninc0 = m.pi_start[base + T] - i0;  // incidences (springs) of the tile
  const int nslot0 = m.pr_nslot[tile];                                  // and the words of their slots
  const int l0 = m.pl_start[tile], nlong0 = m.pl_start[tile + 1] - l0;
  const int nhb0 = m.pr_hub_begin[tile] - e0;  // entries [nhb0, nent0) reach a hub
  const int t0h = m.th_start[tile], nth0 = m.th_start[tile + 1] - t0h;
  const double dt = a.dt;
  const dfloat ddt = df_from_double(a.dt), ddt2 = df_from_double(a.dt / 2.0);
  // hubs this tile owns or reaches, and its copy of each one's state
  __shared__ HubRef s_href[kTileHubs];
  __shared__ int4 s_hmeta[kTileHubs];  // per hub: first partial sum, contributors, slot, moves
  __shared__ __align__(16) unsigned char s_hraw[kTileHubs * (sizeof(HubDF) > sizeof(HubF64) ? sizeof(HubDF) : sizeof(HubF64))];
  HubF64* s_h64 = reinterpret_cast<HubF64*>(s_hraw);
  HubDF* s_hdf = reinterpret_cast<HubDF*>(s_hraw);

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
      if (ok) {
        const int p0 = m.hub_pbase[r.hub], nc = m.hub_pbase[r.hub + 1] - p0, hs = m.hub_slot[r.hub];
        ok &= r.rank < nc && hs >= 0 && hs < m.nslots;
        if (ok) s_hmeta[j] = make_int4(p0, nc, hs, m.moves[hs] == 1);
      }
      nhh += r.idx >= T;
      s_href[j] = r;
    }
    ok &= tot + nhh == hn0 && nrun <= m.df_nrun_max && nsingle <= m.df_nsingle_max;
    ok &= nent0 >= 0 && nent0 <= m.pr_nent_max && nloc0 >= 0 && nloc0 <= nhb0 && nhb0 <= nent0 && ninc0 >= 0 &&
          ninc0 <= nslot0 && nslot0 <= m.pr_ninc_max && nlong0 >= 0 && nlong0 <= m.pr_nlong_max && nb >= 0 &&
          nb <= m.df_nb_max;
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
  const int nslot = plan_ok ? nslot0 : 0;
  const int nlong = plan_ok ? nlong0 : 0, nbt = plan_ok ? nb : 0, nhb = plan_ok ? nhb0 : 0;
  const int nth = plan_ok ? nth0 : 0;
  bool ohub = false;  // the owned bead is a hub: integrated from partial sums, not by its thread
  for (int j = 0; j < nth; ++j) ohub = ohub || s_href[j].idx == tid;
  uint32_t long_bytes = 0;
  if (plan_ok)
    for (int r = 0; r < nrun; ++r) long_bytes += (uint32_t)sizeof(Pos4) * (uint32_t)s_runs[r].z;
  uint32_t hphase = 0;
  // a float64 value as a table word
  auto word = [](double v) -> W {
    if constexpr (kDF) {
      const dfloat d = df_from_double(v);
      return make_float2(d.h, d.l);
    } else {
      return v;
    }
  };
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
    s_rest[i] = word(__ldg(m.pr_rest + e0 + i));
    s_m2k[i] = word(__ldg(m.pr_m2k + e0 + i));
  }
  for (int i = tid; i < nent; i += nthr) {
    uint32_t p = __ldg(m.pr_pos + e0 + i);
    const int ka = (int)(p & 0xffffu), kb = (int)(p >> 16);
    if (ka >= nslot || (kb != 0xffff && kb >= nslot)) {
      atomicOr(a.err, kErrLayout);
      p = 0xffff0000u;  // slot 0 only (a tile with entries has incidences)
    }
    s_pos[i] = p;
  }
  for (int i = tid; i <= T; i += nthr) s_incs[i] = plan_ok ? min(max(m.pi_start[base + i] - i0, 0), ninc) : 0;
  for (int i = tid; i < nlong; i += nthr) {
    // a long bead's slots must lie inside the tile's slot words
    const int bd = min(max(m.pl_list[l0 + i], 0), T - 1);
    int lb = m.pl_base[l0 + i];
    if (lb < 0 || lb + (m.pi_start[base + bd + 1] - m.pi_start[base + bd]) > nslot) {
      atomicOr(a.err, kErrLayout);
      lb = 0;
    }
    s_lng[i] = make_int2(bd, lb);
  }
  for (int i = tid; i < nbt; i += nthr) {
    s_nl[i] = word(m.newlen[b0 + i]);
    s_ol[i] = word(m.oldlen[b0 + i]);
    s_dg[i] = word(m.diag[b0 + i]);
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
          s_tg[k] = word(cilium_target(cl, i, m.midpnt[c]));
          s_bd[k] = word(cl.bending);
        }
      }
      off += nbnd;
    }
  }
  // owned bead state: float64, or cell + pair coordinates and pair velocities and forces
  double x = 0, y = 0, z = 0, vx = 0, vy = 0, vz = 0, fx = 0, fy = 0, fz = 0;
  BeadCoord cx{0, {0.f, 0.f}}, cy{0, {0.f, 0.f}}, cz{0, {0.f, 0.f}};
  dfloat dvx{0.f, 0.f}, dvy{0.f, 0.f}, dvz{0.f, 0.f}, dfx{0.f, 0.f}, dfy{0.f, 0.f}, dfz{0.f, 0.f};
  double ke_coll = 0.0;
  if (oprim) {
    x = m.x[0][oslot];
    y = m.y[0][oslot];
    z = m.z[0][oslot];
    vx = m.vx[oslot];
    vy = m.vy[oslot];
    vz = m.vz[oslot];
    if (a.collide && omoves) ke_coll = bin.collide(x, y, z, vx, vy, vz);  // the beads' collision, folded in
    if constexpr (kDF) {
      cx = coord_from_double(x);
      cy = coord_from_double(y);
      cz = coord_from_double(z);
      dvx = df_from_double(vx);
      dvy = df_from_double(vy);
      dvz = df_from_double(vz);
    }
  }
  // a staged position
  auto stage_f64 = [&](int i, double px, double py, double pz) {
    Pos4 p;
    p.x = px;
    p.y = py;
    p.z = pz;
    p.w = 0.0;
    sp[i] = p;
  };
  auto stage_df = [&](int i, const BeadCoord& qx, const BeadCoord& qy, const BeadCoord& qz) {
    float4 p0, p1;
    pack_coords(qx, qy, qz, p0, p1);
    st[2 * i] = p0;
    st[2 * i + 1] = p1;
  };
  if (tid < nth) {
    // a hub's state at the start of the step, after the beads' collision as
    // its owner applies it (the same arithmetic on the same values)
    const HubRef r = s_href[tid];
    const int hs = m.hub_slot[r.hub];
    double X = m.x[0][hs], Y = m.y[0][hs], Z = m.z[0][hs];
    double VX = m.vx[hs], VY = m.vy[hs], VZ = m.vz[hs];
    if (a.collide && m.moves[hs] == 1) (void)bin.collide(X, Y, Z, VX, VY, VZ);
    if constexpr (kDF) {
      HubDF& H = s_hdf[tid];
      H.x[0] = coord_from_double(X);
      H.x[1] = coord_from_double(Y);
      H.x[2] = coord_from_double(Z);
      H.v[0] = df_from_double(VX);
      H.v[1] = df_from_double(VY);
      H.v[2] = df_from_double(VZ);
      stage_df(r.idx, H.x[0], H.x[1], H.x[2]);
    } else {
      HubF64& H = s_h64[tid];
      H.x[0] = X;
      H.x[1] = Y;
      H.x[2] = Z;
      H.v[0] = VX;
      H.v[1] = VY;
      H.v[2] = VZ;
      stage_f64(r.idx, X, Y, Z);
    }
  }
  __syncwarp();
  if (a.collide) {  // the dissipated-energy bookkeeping of the collided beads
    const double tot = block_sum_f64(ke_coll);
    if (tid == 0 && tot != 0.0) atomicAdd(a.diss, -tot);
  }
  float4* q[2] = {m.q[0], m.q[1]};
  const unsigned nblocks = gridDim.x;
  unsigned barriers = 0;
  int eval = 0;
  bool refreshed = false;

  // own beads into shared memory and the global buffer b
  auto publish = [&](int b) {
    if (oprim && !ohub) {
      if constexpr (kDF) {
        float4 p0, p1;
        pack_coords(cx, cy, cz, p0, p1);
        st[2 * tid] = p0;
        st[2 * tid + 1] = p1;
        q[b][2 * oslot] = p0;
        q[b][2 * oslot + 1] = p1;
      } else {
        stage_f64(tid, x, y, z);
        reinterpret_cast<Pos4*>(q[b])[oslot] = sp[tid];
      }
    }
  };
  // entry i: F = -2k (1 - b / |d|) d, d = x_a - x_b (MDObject::spring, src/libcilia/mdobject.cpp:8-29)
  auto entry = [&](int i) {
    const uint2 c = s_code[i];
    const int ea = (int)(c.x & 0xffffu), eb = (int)(c.x >> 16);
    const int kind = (int)(c.y & 3u), lref = (int)(c.y >> 4);
    const W rl = kind <= MPCD_SPRING_GUARDED ? s_rest[i] : (kind == MPCD_SPRING_BOND ? s_nl[lref] : s_dg[lref]);
    if constexpr (kDF) {
      // the double-float spring of md_df.cu: the difference formed exactly
      // from the cell + offset pairs, |d|^-1 by df_rsqrt, the factor and the
      // force components as pairs (high part, unnormalised low part)
      const DfDiff d = df_diff(st[2 * ea], st[2 * ea + 1], st[2 * eb], st[2 * eb + 1]);
      float2 gx = make_float2(0.f, 0.f), gy = gx, gz = gx;
      if (!(kind == MPCD_SPRING_GUARDED && d.d2.h == 0.0f)) {  // vector-form spring: no force at zero distance
        const float2 k2 = s_m2k[i];
        const dfloat r = df_rsqrt(d.d2);
        const dfloat u = df_two_prod(rl.x, r.h);
        const dfloat w = df_two_sum(1.0f, -u.h);
        const float wl = ((w.l - u.l) - rl.x * r.l) - rl.y * r.h;
        const dfloat f = df_two_prod(k2.x, w.h);
        const float fl = (f.l + k2.x * wl) + k2.y * w.h;
        const dfloat px = df_two_prod(f.h, d.dx.h), py = df_two_prod(f.h, d.dy.h), pz = df_two_prod(f.h, d.dz.h);
        gx = make_float2(px.h, (px.l + f.h * d.dx.l) + fl * d.dx.h);
        gy = make_float2(py.h, (py.l + f.h * d.dy.l) + fl * d.dy.h);
        gz = make_float2(pz.h, (pz.l + f.h * d.dz.l) + fl * d.dz.h);
      }
      const uint32_t p = s_pos[i];
      const int ka = (int)(p & 0xffffu), kb = (int)(p >> 16);
      s_fx[ka] = gx;
      s_fy[ka] = gy;
      s_fz[ka] = gz;
      if (kb != 0xffff) {
        s_fx[kb] = make_float2(-gx.x, -gx.y);
        s_fy[kb] = make_float2(-gy.x, -gy.y);
        s_fz[kb] = make_float2(-gz.x, -gz.y);
      }
    } else {
      const Pos4 pa = sp[ea], pb = sp[eb];
      const double dx = pa.x - pb.x, dy = pa.y - pb.y, dz = pa.z - pb.z;
      const double d2 = dx * dx + dy * dy + dz * dz;
      double gx = 0.0, gy = 0.0, gz = 0.0;
      if (!(kind == MPCD_SPRING_GUARDED && d2 == 0.0)) {  // vector-form spring: no force at zero distance
        const double fac = s_m2k[i] * (1.0 - rl * rsqrt_f64(d2));
        gx = dx * fac;
        gy = dy * fac;
        gz = dz * fac;
      }
      const uint32_t p = s_pos[i];
      const int ka = (int)(p & 0xffffu), kb = (int)(p >> 16);
      s_fx[ka] = gx;
      s_fy[ka] = gy;
      s_fz[ka] = gz;
      if (kb != 0xffff) {
        s_fx[kb] = -gx;
        s_fy[kb] = -gy;
        s_fz[kb] = -gz;
      }
    }
  };
  // a table word, negated when bit 0 of w is set
  auto signed_word = [](W v, uint32_t w) -> W {
    if constexpr (kDF) {
      return (w & 1u) ? make_float2(-v.x, -v.y) : v;
    } else {
      return flip_sign(v, w);
    }
  };
  // running sums: float64, or compensated pairs (h, l)
  struct Acc {
    double d = 0.0;
    float h = 0.f, l = 0.f;
  };
  auto acc_add = [](Acc& s, W v) {
    if constexpr (kDF)
      df_acc(s.h, s.l, v.x, v.y);
    else
      s.d += v;
  };
  auto acc_merge = [&](Acc& s, const Acc& t) {
    if constexpr (kDF)
      df_acc(s.h, s.l, t.h, t.l);
    else
      s.d += t.d;
  };
  auto acc_word = [](const Acc& s) -> W {
    if constexpr (kDF) {
      const dfloat n = df_norm(s.h, s.l);
      return make_float2(n.h, n.l);
    } else {
      return s.d;
    }
  };
  // xor tree over the warp; lane 0 holds the sum in a fixed order
  auto acc_level = [](Acc& s, int o) {
    if constexpr (kDF) {
      const float h = __shfl_xor_sync(0xffffffffu, s.h, o), l = __shfl_xor_sync(0xffffffffu, s.l, o);
      df_acc(s.h, s.l, h, l);
    } else {
      s.d += __shfl_xor_sync(0xffffffffu, s.d, o);
    }
  };
  auto acc_tree = [&](Acc& s) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc_level(s, o);
  };
  // hub j's force from evaluation e: the published partial sums of its
  // contributors (one word per axis) in their order, lane-strided and then by
  // a xor tree; lane 0's sum is the same number in every tile; called by a
  // whole warp
  auto hub_force = [&](int j, int e, W* f) {
    const int p0 = s_hmeta[j].x, nc = s_hmeta[j].y;
    const double* P = m.hubpart + ((size_t)(e & 1) * m.hub_ncon + p0) * 4;
    Acc s[3];
    for (int c = lane; c < nc; c += 32)
      for (int ax = 0; ax < 3; ++ax) {
        const double pv = __ldcg(P + 4 * c + ax);
        if constexpr (kDF)
          acc_add(s[ax], *reinterpret_cast<const float2*>(&pv));
        else
          acc_add(s[ax], pv);
      }
    // the three trees level by level (independent chains side by side)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
      for (int ax = 0; ax < 3; ++ax) acc_level(s[ax], o);
    for (int ax = 0; ax < 3; ++ax) f[ax] = acc_word(s[ax]);
  };
  // before evaluation e >= 1 (after its grid barrier): the last warps, one
  // per hub, advance the tile's copy of hub j with the force of evaluation
  // e - 1, as the Verlet steps of the owned beads, and stage its position,
  // while the other warps evaluate the entries between the tile's own beads
  auto hub_update = [&](int e) {
    const int j = nwarps - 1 - warp;
    if (j < 0 || j >= nth) return;
    const HubRef r = s_href[j];
    W f[3];
    hub_force(j, e - 1, f);
    if (lane == 0) {
      const bool mv = s_hmeta[j].w != 0;
      if constexpr (kDF) {
        HubDF& H = s_hdf[j];
        if (mv)
          for (int ax = 0; ax < 3; ++ax) {
            kick(H.v[ax], dfloat{f[ax].x, f[ax].y}, e == 1 ? ddt2 : ddt);
            coord_kick(H.x[ax], H.v[ax], ddt);
          }
        stage_df(r.idx, H.x[0], H.x[1], H.x[2]);
      } else {
        HubF64& H = s_h64[j];
        if (mv)
          for (int ax = 0; ax < 3; ++ax) {
            H.v[ax] = fma(f[ax], e == 1 ? dt / 2.0 : dt, H.v[ax]);
            H.x[ax] = fma(H.v[ax], dt, H.x[ax]);
          }
        stage_f64(r.idx, H.x[0], H.x[1], H.x[2]);
      }
    }
    // the warp reconverges before the CTA barrier that follows: a barrier
    // reached by lanes 1-31 while lane 0 still works here counted the warp
    // as arrived
    __syncwarp();
  };
  // forces on the owned beads; buffer b holds the other tiles' beads
  auto evaluate = [&](int b) {
    const int ev = eval;
    // from the second evaluation on, the last nth warps advance the hubs'
    // copies (hub_update) while the others (ethr threads) copy the halo and
    // evaluate the entries that do not reach a hub
    const bool hubs_due = ev >= 1 && nth > 0;
    const int ethr = hubs_due ? nthr - 32 * nth : nthr;
    if (hn > 0 && tid < ethr) {
      // the other tiles wrote the buffer through the generic proxy; order
      // those writes (acquired at the barrier) before this thread's bulk reads
      if (tid < nrun) asm volatile("fence.proxy.async.global;" ::: "memory");
      for (int r = tid; r < nrun; r += ethr) {
        const int4 run = s_runs[r];
        bulk_load(st + 2 * (T + run.y), q[b] + 2 * (size_t)run.x, (uint32_t)sizeof(Pos4) * (uint32_t)run.z, hbar);
      }
      for (int i = tid; i < nsingle; i += ethr) {
        const int2 e = s_single[i];
        cp_async16_p(st + 2 * (T + e.y), q[b] + 2 * (size_t)e.x);
        cp_async16_p(st + 2 * (T + e.y) + 1, q[b] + 2 * (size_t)e.x + 1);
      }
    }
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
          const int ia = lb + cl.stride * i, ib = lb + cl.stride * (i + 1);
          if constexpr (kDF) {
            // in pairs, as md_df.cu
            const DfDiff d = df_diff(st[2 * ia], st[2 * ia + 1], st[2 * ib], st[2 * ib + 1]);
            const dfloat tl = df_mul(d.d2, df_rsqrt(d.d2));
            const dfloat tg{s_tg[k].x, s_tg[k].y}, bd{s_bd[k].x, s_bd[k].y}, ol{s_ol[k].x, s_ol[k].y};
            dfloat l = tg;
            if (df_lt(bd, df_abs(df_sub(tg, tl)))) {
              const dfloat t2 = df_lt(tg, tl) ? df_sub(tl, bd) : df_add(tl, bd);
              l = df_sign(df_sub(tg, ol)) * df_sign(df_sub(t2, ol)) > 0 ? t2 : ol;
            }
            const dfloat g = df_sqrt(df_add(dfloat{0.25f, 0.f}, df_mul(dfloat{0.5f, 0.f}, l)));
            s_nl[k] = make_float2(l.h, l.l);
            s_ol[k] = make_float2(l.h, l.l);
            s_dg[k] = make_float2(g.h, g.l);
          } else {
            const double l = cilium_limit(s_tg[k], s_bd[k], s_ol[k], sv64.dist(ia, ib));
            s_nl[k] = l;
            s_ol[k] = l;
            s_dg[k] = sqrt(0.5 * 0.5 + 0.5 * l);
          }
        }
        off += nbnd;
      }
      __syncthreads();
    }
    ++eval;
    if (tid < ethr) {
      // the entries between the tile's own beads, then the halo's
      for (int i = tid; i < nloc; i += ethr) entry(i);
      if (hn > 0) {
        if (long_bytes) {
          if (!mbar_wait(hbar, hphase & 1u, kPairHaloWait)) atomicOr(a.err, kErrBarrier);
          ++hphase;
        }
        cp_async_wait_all_p();
        if (hubs_due)
          asm volatile("bar.sync 1, %0;" ::"r"(ethr) : "memory");  // these warps only
        else
          __syncthreads();  // every thread is here
      }
      for (int i = nloc + tid; i < nhb; i += ethr) entry(i);
    } else {
      hub_update(ev);
    }
    if (nth > 0) {  // the hubs' copies are staged: the entries that reach them
      __syncthreads();
      for (int i = nhb + tid; i < nent; i += nthr) entry(i);
    }
    // the halo region is refilled by the async proxy next substep
    fence_proxy_async_smem();
    __syncthreads();
    // every bead sums its entries in its spring order: a thread per bead and
    // axis, a warp per bead and axis for long lists
    for (int w = tid; w < 3 * T; w += nthr) {
      const int ax = w / T, bd = w - ax * T;  // consecutive threads: consecutive beads
      const int n = s_incs[bd + 1] - s_incs[bd];
      if (n > kPairLong) continue;
      const W* F = (ax == 0 ? s_fx : (ax == 1 ? s_fy : s_fz)) + bd;
      // two chains (alternate springs), then their sum: a fixed order; the
      // j-th slot of bead bd is j * T + bd
      Acc s, t;
      int j = 0;
      for (; j + 1 < n; j += 2) {
        acc_add(s, F[j * T]);
        acc_add(t, F[(j + 1) * T]);
      }
      if (j < n) acc_add(s, F[j * T]);
      acc_merge(s, t);
      s_fs[ax * T + bd] = acc_word(s);
    }
    for (int w = warp; w < 3 * nlong; w += nwarps) {
      const int2 lg = s_lng[w / 3];
      const int bd = lg.x, ax = w % 3;
      const int n = s_incs[bd + 1] - s_incs[bd];
      const W* F = (ax == 0 ? s_fx : (ax == 1 ? s_fy : s_fz)) + lg.y;
      Acc s;
      for (int k = lane; k < n; k += 32) acc_add(s, F[k]);
      acc_tree(s);
      if (lane == 0) s_fs[ax * T + bd] = acc_word(s);
      __syncwarp();
    }
    // the reactions this tile owes each hub: the negated sum of its entries
    // to the hub, in entry order (lane-strided, xor tree), published for the
    // hub's copies after the next grid barrier (by the last warps, beside the
    // sums of the first ones)
    for (int w = nwarps - 1 - warp; w < 3 * nth; w += nwarps) {
      const HubRef r = s_href[w / 3];
      const int ax = w % 3;
      if (r.rank < 0) continue;
      const W* F = ax == 0 ? s_fx : (ax == 1 ? s_fy : s_fz);
      Acc s;
      for (int k = lane; k < r.rn; k += 32) {
        const int ei = __ldg(m.tr_list + r.rs + k);  // an incidence slot of the tile
        if (ei >= 0 && ei < nslot) acc_add(s, signed_word(F[ei], 1u));
      }
      acc_tree(s);
      if (lane == 0) {
        const W v = acc_word(s);
        double* P = m.hubpart + ((size_t)(ev & 1) * m.hub_ncon + s_hmeta[w / 3].x + r.rank) * 4 + ax;
        if constexpr (kDF)
          *reinterpret_cast<float2*>(P) = v;
        else
          *P = v;
      }
      __syncwarp();
    }
    __syncthreads();
    if (oprim) {
      if constexpr (kDF) {
        dfx = dfloat{s_fs[tid].x, s_fs[tid].y};
        dfy = dfloat{s_fs[T + tid].x, s_fs[T + tid].y};
        dfz = dfloat{s_fs[2 * T + tid].x, s_fs[2 * T + tid].y};
      } else {
        fx = s_fs[tid];
        fy = s_fs[T + tid];
        fz = s_fs[2 * T + tid];
      }
    }
  };
  // the grid barrier before every evaluation; the halo's mbarrier is armed
  // with the next copies' bytes before any of them can be issued
  auto barrier = [&]() {
    if (tid == 0 && long_bytes) mbar_arrive_expect_tx(hbar, long_bytes);
    return grid_sync(m.bar, ++barriers * nblocks, a.err);
  };
  // v += F c (c = dt or dt/2), and x += v dt when `drift`
  const bool kicks = omoves && !ohub;  // a hub moves by its copies (hub_update)
  auto verlet = [&](bool half, bool drift) {
    if (!kicks) return;
    if constexpr (kDF) {
      const dfloat c = half ? ddt2 : ddt;
      kick(dvx, dfx, c);
      kick(dvy, dfy, c);
      kick(dvz, dfz, c);
      if (drift) {
        coord_kick(cx, dvx, ddt);
        coord_kick(cy, dvy, ddt);
        coord_kick(cz, dvz, ddt);
      }
    } else {
      const double c = half ? dt / 2.0 : dt;
      vx = fma(fx, c, vx);
      vy = fma(fy, c, vy);
      vz = fma(fz, c, vz);
      if (drift) {
        x = fma(vx, dt, x);
        y = fma(vy, dt, y);
        z = fma(vz, dt, z);
      }
    }
  };

  // md_loop_start: forces at t0, v += F dt/2, x += v dt
  publish(0);
  if (!barrier()) return;
  evaluate(0);
  int cur = 0;
  verlet(true, true);
  publish(cur ^ 1);
  if (!barrier()) return;
  cur ^= 1;
  evaluate(cur);
  // md_loop: v += F dt, x += v dt, forces
  for (int k = 1; k < a.n; ++k) {
    verlet(false, true);
    publish(cur ^ 1);
    if (!barrier()) return;
    cur ^= 1;
    evaluate(cur);
  }
  // md_loop_stop: v += F dt/2, then bin with the next shift
  verlet(true, false);
  if (oprim && !ohub) {
    if constexpr (kDF) {
      x = coord_to_double(cx);
      y = coord_to_double(cy);
      z = coord_to_double(cz);
      vx = df_to_double(dvx);
      vy = df_to_double(dvy);
      vz = df_to_double(dvz);
    }
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
      W f[3];
      hub_force(warp, eval - 1, f);
      if (lane == 0) {
        const int hs = s_hmeta[warp].z;
        const bool mv = s_hmeta[warp].w != 0;
        double X[3], V[3];
        if constexpr (kDF) {
          HubDF& H = s_hdf[warp];
          for (int ax = 0; ax < 3; ++ax) {
            if (mv) kick(H.v[ax], dfloat{f[ax].x, f[ax].y}, ddt2);
            X[ax] = coord_to_double(H.x[ax]);
            V[ax] = df_to_double(H.v[ax]);
          }
        } else {
          HubF64& H = s_h64[warp];
          for (int ax = 0; ax < 3; ++ax) {
            if (mv) H.v[ax] = fma(f[ax], dt / 2.0, H.v[ax]);
            X[ax] = H.x[ax];
            V[ax] = H.v[ax];
          }
        }
        m.x[0][hs] = X[0];
        m.y[0][hs] = X[1];
        m.z[0][hs] = X[2];
        m.vx[hs] = V[0];
        m.vy[hs] = V[1];
        m.vz[hs] = V[2];
        if (mv) {
          if (a.deferred)
            bin.defer(hs, X[0], X[1], X[2], V[0], V[1], V[2]);
          else
            bin(X[0], X[1], X[2], V[0], V[1], V[2]);
        }
      }
      __syncwarp();
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
          if constexpr (kDF) {
            const double l = df_to_double(dfloat{s_nl[k - b0].x, s_nl[k - b0].y});
            m.newlen[k] = l;
            m.oldlen[k] = l;
            m.diag[k] = df_to_double(dfloat{s_dg[k - b0].x, s_dg[k - b0].y});
          } else {
            m.newlen[k] = s_nl[k - b0];
            m.oldlen[k] = s_ol[k - b0];
            m.diag[k] = s_dg[k - b0];
          }
        }
      }
      off += nbnd;
    }
  }
  // switch_logic for the cilia of this tile (the staged positions are the final ones)
  for (int c = c0 + tid; c < c1; c += nthr) {
    if constexpr (kDF)
      cilium_switch(m, a, c, a.t_end, base, svdf);
    else
      cilium_switch(m, a, c, a.t_end, base, sv64);
  }
  __syncthreads();
  if (tid == 0) mbar_inval(hbar);
}

template <bool kDF, typename Bin>
__global__ void __launch_bounds__(512) k_md_pair(MDState m, typename Bin::Cells c, MDStepArgs a) {
  md_pair_body<kDF>(m, a, Bin{c, &a});
}

// the kernel of a layout: float64 (m.pair == 1) or double-float (2)
template <typename Bin>
const void* pair_kernel(const MDState& m) {
  return m.pair == 2 ? (const void*)k_md_pair<true, Bin> : (const void*)k_md_pair<false, Bin>;
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
  const void* k = pair_kernel<Bin>(m);
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
  const void* k = f32cells ? pair_kernel<BinF32>(m) : pair_kernel<BinF64>(m);
  if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, md_pair_threads(m.tile), smem);
  return per_sm * sms;
}

}  // namespace mpcd
