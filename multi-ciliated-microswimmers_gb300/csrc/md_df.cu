// MD substeps of one MPC step for the float64 path, in double-float
// arithmetic on the FP32 pipes.
//
// Same integrator and forces as md_kernels.cu (velocity Verlet of
// src/libcilia/mdobject.cpp:36-72 inside the loop of src/simulation.cpp:217-265;
// springs of src/cilia.cpp:127-239, src/sphere.cpp:87-119, src/clami.cpp:188-198)
// on the same cooperative-grid tile layout (md_plan.cu: a CTA per tile, helper
// slots for long spring lists, halos), with eight lanes per slot (four for
// tiles over 64 slots).  The difference
// is the arithmetic: GB300 issues float64 at a small fraction of its float32
// rate, and the float64 MD kernel spent most of its time on the FP64 pipe.
// Here every bead's position and velocity live in registers as double-float
// pairs (about 48 significand bits) for the whole MPC step; spring forces,
// their sums and the Verlet updates are double-float operations built from
// float adds, multiplies and fused multiply-adds.  The state is read from and
// written back to the float64 arrays once per MPC step.  Rest lengths and
// spring constants come as float pairs prepared on the host.
//
// Each CTA keeps its tile's spring and bond tables in shared memory for the
// whole launch.  Positions are exchanged between tiles through two global
// buffers of pairs (two float4 per bead) after a bounded grid barrier: the
// halo arrives by bulk asynchronous copies (TMA, one per run of consecutive
// slots, completing on an mbarrier) while the lanes work on the springs
// between beads of their own tile, and is waited for (bounded) before the
// springs that reach it.  The partial forces of a bead's helper slots are
// added in a fixed order: by one warp (lane-strided, then a xor tree) for
// long runs, by the primary in slot order for short ones.
//
// The cilia's rest lengths: the beat's target length of every bond is fixed
// during one MPC step's substeps (the midpoint moves after them), so it is
// computed once per launch in float64; the bending-rate limit that uses the
// current bond length runs in pairs at every refresh (every 0.01 time units).
#include <cstdlib>

#include "../../include/mpcd_gpu.h"
#include "df32.cuh"
#include "md_common.cuh"
#include "md_df_coord.cuh"
#include "tma.cuh"

namespace mpcd {

namespace {

constexpr uint32_t kHaloWait = 1u << 22;  // polls of the halo's mbarrier before giving up

// 16-byte asynchronous global -> shared copy through L2 (cp.async.cg)
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Tile-resident spring and bond tables in shared memory.
struct Tables {
  const uint32_t* code;  // other bead | kind << 16 | bond << 18
  const float2* rest;    // static rest length (kinds CONST, GUARDED)
  const float2* m2k;     // -2k
  const float2* nl;      // bonds: current rest length (newlength)
  const float2* dg;      // bonds: diagonal rest length sqrt(0.5^2 + 0.5 newlength)
};

// Force on staged bead `me` from springs [a, b) step LANES (indices local
// to the tile's table).  Per spring, with d = x_me - x_o and rest length b:
// fac = -2k (1 - b / |d|), F += fac d, all in pairs; components accumulate as
// compensated sums (h, l).  kFloat: the difference d is formed exactly as a
// pair and rounded to float, the rest of the spring in float (the split
// arithmetic of the float32 path); the sums stay compensated.
template <int LANES, bool kFloat>
__device__ __forceinline__ void springs_df(const Tables& tb, const float4* st, const float4 m0, const float4 m1, int a,
                                           int b, float& fxh, float& fxl, float& fyh, float& fyl, float& fzh,
                                           float& fzl) {
  for (int s = a; s < b; s += LANES) {
    const uint32_t code = tb.code[s];
    const int o = (int)(code & 0xffffu);
    const int kind = (int)((code >> 16) & 3u);
    const int lref = (int)(code >> 18);
    const float2 b2 = kind <= MPCD_SPRING_GUARDED ? tb.rest[s] : (kind == MPCD_SPRING_BOND ? tb.nl[lref] : tb.dg[lref]);
    const float2 k2 = tb.m2k[s];
    if constexpr (kFloat) {
      const float4 o0 = st[2 * o], o1 = st[2 * o + 1];
      const dfloat ex = coord_diff((float)(cell_x(m1) - cell_x(o1)), m0.x, o0.x, m0.w, o0.w);
      const dfloat ey = coord_diff((float)(cell_y(m1) - cell_y(o1)), m0.y, o0.y, m1.x, o1.x);
      const dfloat ez = coord_diff(__fsub_rn(m1.w, o1.w), m0.z, o0.z, m1.y, o1.y);
      const float dx = ex.h + ex.l, dy = ey.h + ey.l, dz = ez.h + ez.l;
      const float d2 = dx * dx + dy * dy + dz * dz;
      if (kind == MPCD_SPRING_GUARDED && d2 == 0.0f) continue;
      const float fac = k2.x * (1.0f - b2.x * rsqrtf(d2));
      fxh += fac * dx;
      fyh += fac * dy;
      fzh += fac * dz;
      continue;
    }
    const DfDiff d = df_diff(m0, m1, st[2 * o], st[2 * o + 1]);
    if (kind == MPCD_SPRING_GUARDED && d.d2.h == 0.0f) continue;  // vector-form spring: no force at zero distance
    const dfloat r = df_rsqrt(d.d2);
    // w = 1 - b r
    const dfloat u = df_two_prod(b2.x, r.h);
    const dfloat w = df_two_sum(1.0f, -u.h);
    const float wl = ((w.l - u.l) - b2.x * r.l) - b2.y * r.h;
    // fac = -2k w
    const dfloat f = df_two_prod(k2.x, w.h);
    const float fl = (f.l + k2.x * wl) + k2.y * w.h;
    const dfloat gx = df_two_prod(f.h, d.dx.h), gy = df_two_prod(f.h, d.dy.h), gz = df_two_prod(f.h, d.dz.h);
    df_acc(fxh, fxl, gx.h, (gx.l + f.h * d.dx.l) + fl * d.dx.h);
    df_acc(fyh, fyl, gy.h, (gy.l + f.h * d.dy.l) + fl * d.dy.h);
    df_acc(fzh, fzl, gz.h, (gz.l + f.h * d.dz.l) + fl * d.dz.h);
  }
}


// shared-memory layout of one tile
struct DfSmem {
  size_t st, bar, flag, runs, single, code, rest, m2k, nl, ol, dg, tg, bd, part, total;
  __host__ __device__ DfSmem(int T, int hmax, int nsp, int nb, int nrun, int nsingle) {
    size_t o = 0;
    auto take = [&](size_t bytes, size_t align) {
      o = (o + align - 1) / align * align;
      const size_t r = o;
      o += bytes;
      return r;
    };
    st = take(32 * (size_t)(T + hmax), 16);
    bar = take(8, 8);
    flag = take(4, 4);
    runs = take(16 * (size_t)nrun, 16);
    single = take(8 * (size_t)nsingle, 8);
    rest = take(8 * (size_t)nsp, 8);
    m2k = take(8 * (size_t)nsp, 8);
    nl = take(8 * (size_t)nb, 8);
    ol = take(8 * (size_t)nb, 8);
    dg = take(8 * (size_t)nb, 8);
    tg = take(8 * (size_t)nb, 8);
    bd = take(8 * (size_t)nb, 8);
    code = take(4 * (size_t)nsp, 4);
    part = take(24 * (size_t)T, 4);
    total = o;
  }
};

template <int LANES, bool kFloat, typename Bin>
__device__ void md_df_body(const MDState& m, const MDStepArgs& a, Bin bin) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int T = m.tile;
  const DfSmem L(T, m.hmax, m.df_nsp_max, m.df_nb_max, m.df_nrun_max, m.df_nsingle_max);
  float4* st = reinterpret_cast<float4*>(smem + L.st);
  uint32_t* s_code = reinterpret_cast<uint32_t*>(smem + L.code);
  float2* s_rest = reinterpret_cast<float2*>(smem + L.rest);
  float2* s_m2k = reinterpret_cast<float2*>(smem + L.m2k);
  float2* s_nl = reinterpret_cast<float2*>(smem + L.nl);
  float2* s_ol = reinterpret_cast<float2*>(smem + L.ol);
  float2* s_dg = reinterpret_cast<float2*>(smem + L.dg);
  float2* s_tg = reinterpret_cast<float2*>(smem + L.tg);
  float2* s_bd = reinterpret_cast<float2*>(smem + L.bd);
  float* part = reinterpret_cast<float*>(smem + L.part);  // per slot: its lanes' force (6 floats)
  uint64_t* hbar = reinterpret_cast<uint64_t*>(smem + L.bar);  // halo copies' completion
  int* hflag = reinterpret_cast<int*>(smem + L.flag);           // 1: the halo runs are valid
  int4* s_runs = reinterpret_cast<int4*>(smem + L.runs);         // this tile's long halo runs
  int2* s_single = reinterpret_cast<int2*>(smem + L.single);     // and its other halo entries
  const Tables tb{s_code, s_rest, s_m2k, s_nl, s_dg};
  const StageDF sv{st};

  const int tile = blockIdx.x;
  const int base = tile * T;
  const int tid = threadIdx.x;
  const int nthr = blockDim.x;
  // spring lanes: LANES per slot; springs [s0, sm) reach in-tile beads, [sm, s1) the halo
  const int q = tid / LANES, lane = tid % LANES;
  const int slot = base + q;
  const int S0 = m.sp_start[base];
  const int mv = m.moves[slot];
  const int me = mv >= 0 ? m.prim[slot] - base : 0;
  const int s0 = m.sp_start[slot] - S0, sm = m.sp_split[slot] - S0, s1 = m.sp_start[slot + 1] - S0;
  // bead owners: thread tid < T owns slot base + tid
  const int oslot = base + tid;
  const int omv = tid < T ? m.moves[oslot] : -1;
  const bool oprim = omv == 0 || omv == 1, omoves = omv == 1;
  const bool helpers = m.tile_help[tile] != 0;
  // a primary with helpers and its helper slots form a run of 1 + nh slots;
  // runs longer than kTreeRun are summed by a warp, shorter ones by the primary
  constexpr int kTreeRun = 8;
  const int onh = oprim ? m.nhelp[oslot] : 0;
  const int owarps = (T + 31) / 32;  // warps holding the owner threads
  const int h0 = m.halo_start[tile], hn0 = m.halo_start[tile + 1] - h0;
  const int c0 = m.tile_cil[tile], c1 = m.tile_cil[tile + 1];
  const int b0 = m.tile_b0[tile], nb = m.tile_nb[tile];
  const int nsp = m.sp_start[base + T] - S0;
  const dfloat dt = df_from_double(a.dt), dt2 = df_from_double(a.dt / 2.0);

  // halo copies: long runs of consecutive slots by bulk copies (TMA) that
  // complete on an mbarrier, the other entries by per-thread cp.async
  const int r0 = m.halo_run_start[tile], nrun = m.halo_run_start[tile + 1] - r0;
  const int e0 = m.halo_single_start[tile], nsingle = m.halo_single_start[tile + 1] - e0;
  for (int r = tid; r < nrun && nrun <= m.df_nrun_max; r += nthr) s_runs[r] = m.halo_run[r0 + r];
  for (int i = tid; i < nsingle && nsingle <= m.df_nsingle_max; i += nthr) s_single[i] = m.halo_single[e0 + i];
  if (tid == 0) {
    // every copy must stay inside the staged halo and the position buffers,
    // and the copies must cover the halo exactly
    int ok = 1, tot = nsingle;
    for (int r = 0; r < nrun; ++r) {
      const int4 run = m.halo_run[r0 + r];
      ok &= run.z > 0 && run.y >= 0 && run.y + run.z <= m.hmax && run.x >= 0 && run.x + run.z <= m.nslots;
      tot += run.z;
    }
    for (int i = 0; i < nsingle; ++i) {
      const int2 e = m.halo_single[e0 + i];
      ok &= e.y >= 0 && e.y < m.hmax && e.x >= 0 && e.x < m.nslots;
    }
    ok &= tot == hn0 && nrun <= m.df_nrun_max && nsingle <= m.df_nsingle_max;
    if (!ok) atomicOr(a.err, kErrLayout);
    *hflag = ok;
    mbar_init(hbar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  const bool halo_ok = *hflag != 0;  // no halo copies (and an error) for an inconsistent plan
  const int hn = halo_ok ? hn0 : 0;
  uint32_t long_bytes = 0;
  if (halo_ok)
    for (int r = 0; r < nrun; ++r) long_bytes += 32u * (uint32_t)s_runs[r].z;
  uint32_t hphase = 0;
  // tile-resident tables
  for (int i = tid; i < nsp; i += nthr) {
    s_code[i] = __ldg(m.sp_code + S0 + i);
    s_rest[i] = __ldg(m.sp_rest2 + S0 + i);
    s_m2k[i] = __ldg(m.sp_m2k2 + S0 + i);
  }
  for (int i = tid; i < nb; i += nthr) {
    const dfloat n = df_from_double(m.newlen[b0 + i]), o = df_from_double(m.oldlen[b0 + i]);
    const dfloat g = df_from_double(m.diag[b0 + i]);
    s_nl[i] = make_float2(n.h, n.l);
    s_ol[i] = make_float2(o.h, o.l);
    s_dg[i] = make_float2(g.h, g.l);
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
        const dfloat t = df_from_double(cilium_target(cl, i, m.midpnt[c]));
        const dfloat bd = df_from_double(cl.bending);
        s_tg[k] = make_float2(t.h, t.l);
        s_bd[k] = make_float2(bd.h, bd.l);
      }
      off += nbnd;
    }
  }
  BeadCoord x{0, {0.f, 0.f}}, y{0, {0.f, 0.f}}, z{0, {0.f, 0.f}};
  dfloat vx{0.f, 0.f}, vy{0.f, 0.f}, vz{0.f, 0.f};
  dfloat fx{0.f, 0.f}, fy{0.f, 0.f}, fz{0.f, 0.f};
  double ke_coll = 0.0;
  if (oprim) {
    const double X = m.x[0][oslot], Y = m.y[0][oslot], Z = m.z[0][oslot];
    double VX = m.vx[oslot], VY = m.vy[oslot], VZ = m.vz[oslot];
    if (a.collide && omoves) ke_coll = bin.collide(X, Y, Z, VX, VY, VZ);  // the beads' collision, folded in
    x = coord_from_double(X);
    y = coord_from_double(Y);
    z = coord_from_double(Z);
    vx = df_from_double(VX);
    vy = df_from_double(VY);
    vz = df_from_double(VZ);
  }
  if (a.collide) {  // the dissipated-energy bookkeeping of the collided beads
    const double tot = block_sum_f64(ke_coll);
    if (tid == 0 && tot != 0.0) atomicAdd(a.diss, -tot);
  }
  const unsigned nblocks = gridDim.x;
  unsigned barriers = 0;
  int eval = 0;
  bool refreshed = false;

  // own beads into shared memory and the global pair buffer b
  auto publish = [&](int b) {
    if (oprim) {
      float4 p0, p1;
      pack_coords(x, y, z, p0, p1);
      st[2 * tid] = p0;
      st[2 * tid + 1] = p1;
      m.q[b][2 * oslot] = p0;
      m.q[b][2 * oslot + 1] = p1;
    }
  };
  // forces on the owned beads; buffer b holds the other tiles' beads
  auto evaluate = [&](int b) {
    // other tiles' beads: one bulk asynchronous copy (TMA) per run of
    // consecutive slots, completing on the mbarrier; waited for before the
    // halo springs
    if (hn > 0) {
      // the other tiles wrote the buffer through the generic proxy; order
      // those writes (acquired at the barrier) before this thread's bulk reads
      if (tid < nrun) asm volatile("fence.proxy.async.global;" ::: "memory");
      for (int r = tid; r < nrun; r += nthr) {
        const int4 run = s_runs[r];
        bulk_load(st + 2 * (T + run.y), m.q[b] + 2 * (size_t)run.x, 32u * (uint32_t)run.z, hbar);
      }
      for (int i = tid; i < nsingle; i += nthr) {
        const int2 e = s_single[i];
        cp_async16(st + 2 * (T + e.y), m.q[b] + 2 * (size_t)e.x);
        cp_async16(st + 2 * (T + e.y) + 1, m.q[b] + 2 * (size_t)e.x + 1);
      }
    }
    if (c1 > c0 && refresh_due(a, eval)) {
      // Cilia::length (src/cilia.cpp:79-121) for every refreshed bond, in pairs
      refreshed = true;
      int off = 0;
      for (int c = c0; c < c1; ++c) {
        const CiliumDev cl = m.cil[c];
        const int nbnd = cl.len - cl.num_anker;
        const int w = tid - off;
        if (w >= 0 && w < nbnd) {
          const int i = cl.num_anker - 1 + w;
          const int k = cl.bond_base + i - b0;
          const int l0 = cl.slot0 - base;
          const int ia = l0 + cl.stride * i, ib = l0 + cl.stride * (i + 1);
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
        }
        off += nbnd;
      }
      __syncthreads();
    }
    ++eval;
    float axh = 0.f, axl = 0.f, ayh = 0.f, ayl = 0.f, azh = 0.f, azl = 0.f;
    float4 m0 = make_float4(0.f, 0.f, 0.f, 0.f), m1 = m0;
    if (mv >= 0) {
      m0 = st[2 * me];
      m1 = st[2 * me + 1];
      springs_df<LANES, kFloat>(tb, st, m0, m1, s0 + lane, sm, axh, axl, ayh, ayl, azh, azl);
    }
    if (hn > 0) {
      if (long_bytes) {
        if (!mbar_wait(hbar, hphase & 1u, kHaloWait)) atomicOr(a.err, kErrBarrier);
        ++hphase;
      }
      cp_async_wait_all();
      __syncthreads();
    }
    if (mv >= 0) springs_df<LANES, kFloat>(tb, st, m0, m1, sm + lane, s1, axh, axl, ayh, ayl, azh, azl);
    // the halo region is refilled by the async proxy next substep
    fence_proxy_async_smem();
    // fixed-order combination of the four lanes
#pragma unroll
    for (int o = 1; o < LANES; o <<= 1) {
      const float bxh = __shfl_xor_sync(0xffffffffu, axh, o), bxl = __shfl_xor_sync(0xffffffffu, axl, o);
      const float byh = __shfl_xor_sync(0xffffffffu, ayh, o), byl = __shfl_xor_sync(0xffffffffu, ayl, o);
      const float bzh = __shfl_xor_sync(0xffffffffu, azh, o), bzl = __shfl_xor_sync(0xffffffffu, azl, o);
      df_acc(axh, axl, bxh, bxl);
      df_acc(ayh, ayl, byh, byl);
      df_acc(azh, azl, bzh, bzl);
    }
    if (lane == 0) {
      float* pp = part + 6 * q;
      pp[0] = axh;
      pp[1] = axl;
      pp[2] = ayh;
      pp[3] = ayl;
      pp[4] = azh;
      pp[5] = azl;
    }
    __syncthreads();
    if (helpers && tid < 32 * owarps) {
      // long runs: the warp holding the primary's owner thread adds the run's
      // slot sums, lane-strided and then by a xor tree -- a fixed order
      const int lane32 = tid & 31;
      unsigned runs = __ballot_sync(0xffffffffu, onh + 1 > kTreeRun);
      while (runs) {
        const int src = __ffs(runs) - 1;
        runs &= runs - 1;
        const int p = (tid & ~31) + src;
        const int len = 1 + __shfl_sync(0xffffffffu, onh, src);
        float gxh = 0.f, gxl = 0.f, gyh = 0.f, gyl = 0.f, gzh = 0.f, gzl = 0.f;
        for (int k = lane32; k < len; k += 32) {
          const float* ph = part + 6 * (p + k);
          df_acc(gxh, gxl, ph[0], ph[1]);
          df_acc(gyh, gyl, ph[2], ph[3]);
          df_acc(gzh, gzl, ph[4], ph[5]);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const float bxh = __shfl_xor_sync(0xffffffffu, gxh, o), bxl = __shfl_xor_sync(0xffffffffu, gxl, o);
          const float byh = __shfl_xor_sync(0xffffffffu, gyh, o), byl = __shfl_xor_sync(0xffffffffu, gyl, o);
          const float bzh = __shfl_xor_sync(0xffffffffu, gzh, o), bzl = __shfl_xor_sync(0xffffffffu, gzl, o);
          df_acc(gxh, gxl, bxh, bxl);
          df_acc(gyh, gyl, byh, byl);
          df_acc(gzh, gzl, bzh, bzl);
        }
        if (lane32 == src) {
          fx = df_norm(gxh, gxl);
          fy = df_norm(gyh, gyl);
          fz = df_norm(gzh, gzl);
        }
      }
    }
    if (oprim && onh > 0 && onh + 1 <= kTreeRun) {  // short runs, in slot order
      const float* pp = part + 6 * tid;
      float gxh = pp[0], gxl = pp[1], gyh = pp[2], gyl = pp[3], gzh = pp[4], gzl = pp[5];
      for (int k = 1; k <= onh; ++k) {
        const float* ph = pp + 6 * k;
        df_acc(gxh, gxl, ph[0], ph[1]);
        df_acc(gyh, gyl, ph[2], ph[3]);
        df_acc(gzh, gzl, ph[4], ph[5]);
      }
      fx = df_norm(gxh, gxl);
      fy = df_norm(gyh, gyl);
      fz = df_norm(gzh, gzl);
    }
    if (oprim && onh == 0) {
      const float* pp = part + 6 * tid;
      fx = df_norm(pp[0], pp[1]);
      fy = df_norm(pp[2], pp[3]);
      fz = df_norm(pp[4], pp[5]);
    }
  };
  // the grid barrier before every evaluation; the halo's mbarrier is armed
  // with the next copies' bytes before any of them can be issued
  auto barrier = [&]() {
    if (tid == 0 && long_bytes) mbar_arrive_expect_tx(hbar, long_bytes);
    return grid_sync(m.bar, ++barriers * nblocks, a.err);
  };

  // md_loop_start: forces at t0, v += F dt/2, x += v dt
  publish(0);
  if (!barrier()) return;
  evaluate(0);
  int cur = 0;
  if (omoves) {
    kick(vx, fx, dt2);
    kick(vy, fy, dt2);
    kick(vz, fz, dt2);
    coord_kick(x, vx, dt);
    coord_kick(y, vy, dt);
    coord_kick(z, vz, dt);
  }
  publish(cur ^ 1);
  if (!barrier()) return;
  cur ^= 1;
  evaluate(cur);
  // md_loop: v += F dt, x += v dt, forces
  for (int k = 1; k < a.n; ++k) {
    if (omoves) {
      kick(vx, fx, dt);
      kick(vy, fy, dt);
      kick(vz, fz, dt);
      coord_kick(x, vx, dt);
      coord_kick(y, vy, dt);
      coord_kick(z, vz, dt);
    }
    publish(cur ^ 1);
    if (!barrier()) return;
    cur ^= 1;
    evaluate(cur);
  }
  // md_loop_stop: v += F dt/2, then bin with the next shift
  if (omoves) {
    kick(vx, fx, dt2);
    kick(vy, fy, dt2);
    kick(vz, fz, dt2);
  }
  if (oprim) {
    const double X = coord_to_double(x), Y = coord_to_double(y), Z = coord_to_double(z);
    const double VX = df_to_double(vx), VY = df_to_double(vy), VZ = df_to_double(vz);
    m.x[0][oslot] = X;
    m.y[0][oslot] = Y;
    m.z[0][oslot] = Z;
    m.vx[oslot] = VX;
    m.vy[oslot] = VY;
    m.vz[oslot] = VZ;
    if (omoves) {
      if (a.deferred)
        bin.defer(oslot, X, Y, Z, VX, VY, VZ);
      else
        bin(X, Y, Z, VX, VY, VZ);
    }
  }
  // refreshed bonds back to float64
  if (refreshed) {
    int off = 0;
    for (int c = c0; c < c1; ++c) {
      const CiliumDev cl = m.cil[c];
      const int nbnd = cl.len - cl.num_anker;
      const int w = tid - off;
      if (w >= 0 && w < nbnd) {
        const int k = cl.bond_base + cl.num_anker - 1 + w;
        const double l = df_to_double(dfloat{s_nl[k - b0].x, s_nl[k - b0].y});
        m.newlen[k] = l;
        m.oldlen[k] = l;
        m.diag[k] = df_to_double(dfloat{s_dg[k - b0].x, s_dg[k - b0].y});
      }
      off += nbnd;
    }
  }
  // switch_logic for the cilia of this tile (the staged positions are the final ones)
  for (int c = c0 + tid; c < c1; c += nthr) cilium_switch(m, a, c, a.t_end, base, sv);
  __syncthreads();
  if (tid == 0) mbar_inval(hbar);
}

template <int LANES, bool kFloat, typename Bin>
__global__ void __launch_bounds__(512) k_md_df(MDState m, typename Bin::Cells c, MDStepArgs a) {
  md_df_body<LANES, kFloat>(m, a, Bin{c, &a});
}

// the kernel for a layout: lanes per slot, double-float (m.df == 1) or float springs (2)
template <typename Bin>
const void* df_kernel(const MDState& m, int lanes) {
  const bool fl = m.df == 2;
  if (lanes == 8) return fl ? (const void*)k_md_df<8, true, Bin> : (const void*)k_md_df<8, false, Bin>;
  if (lanes == 2) return fl ? (const void*)k_md_df<2, true, Bin> : (const void*)k_md_df<2, false, Bin>;
  return fl ? (const void*)k_md_df<4, true, Bin> : (const void*)k_md_df<4, false, Bin>;
}

}  // namespace

// eight lanes per slot when the tile allows it (more warps in flight), else
// four, and two for the widest tiles (at most 512 threads per CTA)
int md_df_lanes(int tile) {
  static const int forced = [] {
    const char* env = std::getenv("MPCD_MD_DF_LANES");  // 4 or 8
    return env ? std::atoi(env) : 0;
  }();
  if (tile > 128) return 2;
  if (forced == 4 || (forced == 8 && tile <= 64)) return forced;
  return tile <= 64 ? 8 : 4;
}

namespace {

size_t md_df_smem(const MDState& m) {
  return DfSmem(m.tile, m.hmax, m.df_nsp_max, m.df_nb_max, m.df_nrun_max, m.df_nsingle_max).total;
}

template <typename Bin>
int launch_df(const MDState& m, const typename Bin::Cells& c, const MDStepArgs& a, cudaStream_t s, cudaError_t* st) {
  if (m.nslots == 0 || m.ntiles == 0) return 0;
  cudaMemsetAsync(m.bar.count, 0, 2 * sizeof(unsigned), s);  // count and gen are adjacent
  MDState mm = m;
  typename Bin::Cells cc = c;
  MDStepArgs aa = a;
  void* args[] = {&mm, &cc, &aa};
  const size_t smem = md_df_smem(m);
  const int lanes = md_df_lanes(m.tile);
  const void* k = df_kernel<Bin>(m, lanes);
  if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  *st = cudaLaunchCooperativeKernel(k, dim3(m.ntiles), dim3(lanes * m.tile), args, smem, s);
  return 1;
}

}  // namespace

int launch_md_df_f64cells(const MDState& m, const CellsF64& c, const MDStepArgs& a, cudaStream_t s, cudaError_t* st) {
  return launch_df<BinF64>(m, c, a, s, st);
}

int launch_md_df_f32cells(const MDState& m, const CellsF32& c, const MDStepArgs& a, cudaStream_t s, cudaError_t* st) {
  return launch_df<BinF32>(m, c, a, s, st);
}

int md_df_max_coresident_blocks(const MDState& m, int f32cells) {
  int dev = 0, sms = 0, per_sm = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t smem = md_df_smem(m);
  if (smem > (size_t)optin) return 0;
  const int lanes = md_df_lanes(m.tile);
  const void* k = f32cells ? df_kernel<BinF32>(m, lanes) : df_kernel<BinF64>(m, lanes);
  if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, lanes * m.tile, smem);
  return per_sm * sms;
}

}  // namespace mpcd
