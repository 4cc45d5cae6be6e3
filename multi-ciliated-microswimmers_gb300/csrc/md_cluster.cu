// Split-precision MD substeps on one thread-block cluster per swimmer.
//
// The same physics as md_kernels.cu (src/libcilia/mdobject.cpp:36-72,
// src/cilia.cpp:79-239, src/sphere.cpp:87-119, src/clami.cpp:188-198,
// src/simulation.cpp:217-265), laid out for a cluster of up to 16 CTAs:
//  - every CTA owns one tile of bead slots (two lanes per slot) and keeps its
//    springs, its cilia's bond tables and two buffers of positions (float
//    hi/lo pairs) in shared memory for the whole launch;
//  - beads of other CTAs that a tile's springs reach are read through
//    distributed shared memory from the owner's current position buffer;
//  - one hardware cluster barrier per substep orders the position writes of
//    substep k before the reads of substep k+1 (the buffers alternate, so
//    nobody overwrites what another CTA may still be reading).
// Nothing goes through global memory between substeps.  State (positions,
// velocities) and the integration stay float64 in registers.
#include <cooperative_groups.h>

#include "batch_internal.h"
#include "engine_internal.h"
#include "fluid_device.cuh"

namespace cg = cooperative_groups;

namespace mpcd {

namespace {


// Cilia::length(i) (src/cilia.cpp:79-121) in float arithmetic; cp = (num_anker,
// rodlength, beatstrength, bending) of the cilium
__device__ float cl_cilium_length(const float4 cp, int i, float midpnt, float oldlen, float tl) {
  const float bondlength = 0.5f, beat = cp.z, bend = cp.w;
  float l;
  if ((float)i < midpnt - 2.0f) {
    const float base = 1.0f - ((float)i - cp.x - 1.0f) / (cp.y - cp.x - 1.0f);
    l = bondlength + beat * (base * base * sqrtf(base)) * 0.5f * (1.0f - 1.0f / (midpnt - (float)i - 1.0f));
  } else {
    const float di = (float)i - midpnt;
    l = bondlength - 2.0f * beat / (di * di + 1.0f);
  }
  if (fabsf(l - tl) > bend) {
    tl = tl + bend - 2.0f * bend * (l < tl ? 1.0f : 0.0f);
    l = (l - oldlen) * (tl - oldlen) > 0.0f ? tl : oldlen;
  }
  return l;
}

// one position buffer: six float arrays of length np (hi x,y,z then lo x,y,z)
// One position buffer of np beads: (hi x, hi y, hi z, lo x) as float4 and
// (lo y, lo z) as float2, so that a neighbour costs two shared loads.
struct PBuf {
  float4* p4;
  float2* p2;
  __device__ void put(int i, const float* h, const float* l) const {
    p4[i] = make_float4(h[0], h[1], h[2], l[0]);
    p2[i] = make_float2(l[1], l[2]);
  }
  // x_i - x_j from the hi/lo pairs, in float
  __device__ void diff(int i, int j, float& dx, float& dy, float& dz) const {
    const float4 a = p4[i], b = p4[j];
    const float2 c = p2[i], d = p2[j];
    dx = (a.x - b.x) + (a.w - b.w);
    dy = (a.y - b.y) + (c.x - d.x);
    dz = (a.z - b.z) + (c.y - d.y);
  }
  __device__ float dist(int i, int j) const {
    float dx, dy, dz;
    diff(i, j, dx, dy, dz);
    return sqrtf(dx * dx + dy * dy + dz * dz);
  }
};

// positions staged per CTA: the tile's slots and its halo, rounded up to an
// even count so that every buffer's float4 part stays 16-byte aligned
__host__ __device__ inline int cl_np(int tile, int hmax) { return (tile + hmax + 1) & ~1; }


// Shared memory of one CTA: nsp_max springs (CSR by slot), nbond_max entries
// of the bond tables.
struct ClusterLayout {
  int np, nsp_max, nbond_max;  // np even (cl_np)
  int nbuf;  // position buffers: 2 (one cluster barrier per substep) or 1 (two, less shared memory)
  __host__ __device__ int max_cilia() const { return nbond_max / 2 + 1; }
  __host__ __device__ int nsp2() const { return (nsp_max + 1) & ~1; }
  __host__ __device__ size_t bytes(int T) const {
    size_t b = (size_t)nbuf * 6 * sizeof(float) * (size_t)np;  // position buffers
    b += (size_t)nsp2() * (sizeof(uint32_t) + 2 * sizeof(float));  // springs: word, (rest, -2k)
    b += (size_t)nbond_max * 3 * sizeof(float);                      // bond tables
    b = (b + 15) & ~(size_t)15;
    b += (size_t)nbond_max * sizeof(int4);                      // refresh entries
    b += (size_t)max_cilia() * (sizeof(float4) + sizeof(float));  // cilium parameters, midpoints
    b = (b + 15) & ~(size_t)15;
    b += 3 * sizeof(float) * (size_t)T;                         // helper partial forces
    return b;
  }
};

// The MD of one swimmer on one cluster; `tile` is this CTA's tile (the
// cluster's CTAs hold consecutive tiles).  Bin::kCollide: the beads first
// take the SRD collision of the current step (bead_collide folded in).
template <int kCLanes, typename Bin>
__device__ __forceinline__ void md_cluster_body(const MDState& m, const MDStepArgs& a, const Bin& bin,
                                                const ClusterLayout& lay, const int tile) {
  extern __shared__ __align__(16) unsigned char smem[];
  cg::cluster_group cluster = cg::this_cluster();
  const int T = m.tile;
  const int np = lay.np;
  const int first_tile = tile - (int)cluster.block_rank();
  const int base = tile * T;
  // carve shared memory
  unsigned char* ptr = smem;
  unsigned char* const pbase = ptr;  // buffer b at pbase + b * 24 * np bytes
  const int nbuf = lay.nbuf;
  auto buf = [&](int b) {
    unsigned char* q = pbase + (size_t)(nbuf == 2 ? b : 0) * 24 * np;
    return PBuf{reinterpret_cast<float4*>(q), reinterpret_cast<float2*>(q + 16 * (size_t)np)};
  };
  ptr += (size_t)nbuf * 24 * (size_t)np;
  float2* srk = reinterpret_cast<float2*>(ptr);                  // (rest, -2k) per spring
  uint32_t* sw = reinterpret_cast<uint32_t*>(srk + lay.nsp2());  // other | bond entry << 16
  ptr = reinterpret_cast<unsigned char*>(sw + lay.nsp2());
  float* bnew = reinterpret_cast<float*>(ptr);
  float* bold = bnew + lay.nbond_max;
  float* bdiag = bold + lay.nbond_max;
  ptr = reinterpret_cast<unsigned char*>(((uintptr_t)(bdiag + lay.nbond_max) + 15) & ~(uintptr_t)15);
  int4* rf = reinterpret_cast<int4*>(ptr);  // per bond: (slot i, slot i+1, position i, cilium), x < 0 unused
  float4* cpar = reinterpret_cast<float4*>(rf + lay.nbond_max);
  float* cmid = reinterpret_cast<float*>(cpar + lay.max_cilia());
  ptr = reinterpret_cast<unsigned char*>(cmid + lay.max_cilia());
  float* part = reinterpret_cast<float*>(((uintptr_t)ptr + 15) & ~(uintptr_t)15);

  // per-tile constants
  const int c0 = m.tile_cil[tile], c1 = m.tile_cil[tile + 1];
  const int bond0 = c1 > c0 ? m.cil[c0].bond_base : 0;
  const int nbond = c1 > c0 ? m.cil[c1 - 1].bond_base + m.cil[c1 - 1].len - bond0 : 0;
  const int h0 = m.halo_start[tile], hn = m.halo_start[tile + 1] - h0;
  const int q = threadIdx.x / kCLanes, lane = threadIdx.x % kCLanes;  // kCLanes lanes per slot
  const int slot = base + q;
  const bool valid = q < T;
  // stage the tile's springs (CSR by slot)
  const int sp0 = m.sp_start[base], sp1 = m.sp_start[base + T];
  if (sp1 - sp0 > lay.nsp_max) {  // layout smaller than the tile needs: no springs, and say so
    if (threadIdx.x == 0) atomicOr(a.err, kErrLayout);
  } else {
    for (int s = sp0 + (int)threadIdx.x; s < sp1; s += blockDim.x) {
      const int k = s - sp0;
      const int kind = m.sp_kind[s] & 3;
      // BOND/DIAG springs carry their bond-table entry in the high half
      const uint32_t bl = kind >= 2 ? (uint32_t)(m.sp_ref[s] - bond0) : 0u;
      sw[k] = (uint32_t)m.sp_local[s] | (bl << 16);
      srk[k] = make_float2((float)m.sp_rest[s], (float)m.sp_m2k[s]);
    }
  }
  const int s0 = valid && sp1 - sp0 <= lay.nsp_max ? m.sp_start[slot] - sp0 : 0;
  const int s1 = valid && sp1 - sp0 <= lay.nsp_max ? m.sp_start[slot + 1] - sp0 : 0;
  // group boundaries of this slot's list (the planner sorts it by spring_group):
  // CONST [s0, g1), CONST owed to a hub [g1, g2), GUARDED [g2, g3), BOND [g3, g4), DIAG [g4, s1)
  int g1 = s0, g2 = s0, g3 = s0, g4 = s0;  // ends of groups 0..3; group 4 ends at s1
  for (int s = s0; s < s1; ++s) {
    const int grp = spring_group(m.sp_kind[sp0 + s]);
    g1 += grp < 1;
    g2 += grp < 2;
    g3 += grp < 3;
    g4 += grp < 4;
  }
  for (int k = threadIdx.x; k < nbond; k += blockDim.x) {
    bnew[k] = (float)m.newlen[bond0 + k];
    bold[k] = (float)m.oldlen[bond0 + k];
    bdiag[k] = (float)m.diag[bond0 + k];
    rf[k] = make_int4(-1, 0, 0, 0);
  }
  __syncthreads();
  // refresh entries: the driven bonds num_anker-1 .. rodlength-2 of every cilium
  for (int c = c0 + (int)threadIdx.x; c < c1; c += (int)blockDim.x) {
    const CiliumDev cl = m.cil[c];
    const int cc = c - c0;
    cpar[cc] = make_float4((float)cl.num_anker, (float)cl.len, (float)cl.beatstrength, (float)cl.bending);
    cmid[cc] = (float)m.midpnt[c];
    const int l0 = cl.slot0 - base, sd = cl.stride;
    for (int i = cl.num_anker - 1; i <= cl.len - 2; ++i)
      rf[cl.bond_base - bond0 + i] = make_int4(l0 + sd * i, l0 + sd * (i + 1), i, cc);
  }
  const int mv = valid ? m.moves[slot] : -1;
  const bool moves = mv == 1;
  const bool primary = mv == 0 || mv == 1;
  const int me = valid && mv >= 0 ? m.prim[slot] - base : 0;
  const int nh = primary ? m.nhelp[slot] : 0;
  const bool helpers = m.tile_help[tile] != 0;
  const int hub_local = m.tile_react[tile];
  const float fdt = (float)a.dt;
  // position as float hi + lo (x = hi + lo to ~48 bits), velocity and force float
  float xh[3] = {0.f, 0.f, 0.f}, xl[3] = {0.f, 0.f, 0.f}, v[3] = {0.f, 0.f, 0.f};
  float fx = 0.f, fy = 0.f, fz = 0.f;
  double X[3] = {0.0, 0.0, 0.0};
  if (primary) {
    X[0] = m.x[0][slot];
    X[1] = m.y[0][slot];
    X[2] = m.z[0][slot];
    for (int d = 0; d < 3; ++d) {
      xh[d] = (float)X[d];
      xl[d] = (float)(X[d] - (double)xh[d]);
    }
    v[0] = (float)m.vx[slot];
    v[1] = (float)m.vy[slot];
    v[2] = (float)m.vz[slot];
  }
  if constexpr (Bin::kCollide) {  // MDObject beads in MPCD::next_tstep (src/libcilia/mpcd.cpp:140-247)
    double ke = 0.0;
    if (moves && lane == 0) ke = bin.collide(X, v);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ke += __shfl_xor_sync(0xffffffffu, ke, o);
    if ((threadIdx.x & 31) == 0 && ke != 0.0) bin.add_diss(-ke);
  }
  if (primary && lane == 0) buf(0).put(q, xh, xl);
  int cur = 0;
  int eval = 0;  // index of the force evaluation within this MPC step
  cluster.sync();  // every CTA's first buffer is filled

  auto evaluate = [&]() {
    const PBuf B = buf(cur);
    // halo: beads of other CTAs, from their current buffer
    for (int i = threadIdx.x; i < hn; i += blockDim.x) {
      const int gs = m.halo[h0 + i];
      const int r = gs / T - first_tile, j = gs % T;
      const float4* rp4 = cluster.map_shared_rank(B.p4, r);
      const float2* rp2 = cluster.map_shared_rank(B.p2, r);
      B.p4[T + i] = rp4[j];
      B.p2[T + i] = rp2[j];
    }
    __syncthreads();
    const bool due = (a.refresh[eval >> 6] >> (eval & 63)) & 1ull;  // refresh (src/cilia.cpp:206-215)
    ++eval;
    if (c1 > c0 && due) {
      for (int k = threadIdx.x; k < nbond; k += blockDim.x) {
        const int4 e = rf[k];
        if (e.x < 0) continue;
        const float l = cl_cilium_length(cpar[e.w], e.z, cmid[e.w], bold[k], B.dist(e.x, e.y));
        bnew[k] = l;
        bold[k] = l;
        bdiag[k] = sqrtf(0.25f + 0.5f * l);
      }
      __syncthreads();
    }
    float ax = 0.f, ay = 0.f, az = 0.f;
    float rx = 0.f, ry = 0.f, rz = 0.f;  // reactions owed to the tile's hub
    if (mv >= 0) {
      // one loop per spring group: no per-spring dispatch on the kind
      const float4 m4 = B.p4[me];
      const float2 m2 = B.p2[me];
      auto geo = [&](int o, float& dx, float& dy, float& dz) {
        const float4 b4 = B.p4[o];
        const float2 b2 = B.p2[o];
        dx = (m4.x - b4.x) + (m4.w - b4.w);
        dy = (m4.y - b4.y) + (m2.x - b2.x);
        dz = (m4.z - b4.z) + (m2.y - b2.y);
      };
#pragma unroll 2
      for (int s = s0 + lane; s < g1; s += kCLanes) {  // CONST
        const float2 rk = srk[s];
        float dx, dy, dz;
        geo((int)sw[s], dx, dy, dz);
        const float fac = rk.y * (1.0f - rk.x * rsqrtf(dx * dx + dy * dy + dz * dz));
        ax = fmaf(dx, fac, ax);
        ay = fmaf(dy, fac, ay);
        az = fmaf(dz, fac, az);
      }
      for (int s = g1 + lane; s < g2; s += kCLanes) {  // CONST, reaction owed to the hub
        const float2 rk = srk[s];
        float dx, dy, dz;
        geo((int)sw[s], dx, dy, dz);
        const float fac = rk.y * (1.0f - rk.x * rsqrtf(dx * dx + dy * dy + dz * dz));
        ax = fmaf(dx, fac, ax);
        ay = fmaf(dy, fac, ay);
        az = fmaf(dz, fac, az);
        rx = fmaf(-dx, fac, rx);
        ry = fmaf(-dy, fac, ry);
        rz = fmaf(-dz, fac, rz);
      }
      for (int s = g2 + lane; s < g3; s += kCLanes) {  // GUARDED: no force at zero distance
        const float2 rk = srk[s];
        float dx, dy, dz;
        geo((int)sw[s], dx, dy, dz);
        const float d2 = dx * dx + dy * dy + dz * dz;
        const float fac = d2 == 0.0f ? 0.0f : rk.y * (1.0f - rk.x * rsqrtf(d2));
        ax = fmaf(dx, fac, ax);
        ay = fmaf(dy, fac, ay);
        az = fmaf(dz, fac, az);
      }
#pragma unroll 2
      for (int s = g3 + lane; s < g4; s += kCLanes) {  // BOND: active rest length
        const uint32_t w = sw[s];
        const float b = bnew[w >> 16];
        float dx, dy, dz;
        geo((int)(w & 0xffffu), dx, dy, dz);
        const float fac = srk[s].y * (1.0f - b * rsqrtf(dx * dx + dy * dy + dz * dz));
        ax = fmaf(dx, fac, ax);
        ay = fmaf(dy, fac, ay);
        az = fmaf(dz, fac, az);
      }
#pragma unroll 2
      for (int s = g4 + lane; s < s1; s += kCLanes) {  // DIAG
        const uint32_t w = sw[s];
        const float b = bdiag[w >> 16];
        float dx, dy, dz;
        geo((int)(w & 0xffffu), dx, dy, dz);
        const float fac = srk[s].y * (1.0f - b * rsqrtf(dx * dx + dy * dy + dz * dz));
        ax = fmaf(dx, fac, ax);
        ay = fmaf(dy, fac, ay);
        az = fmaf(dz, fac, az);
      }
    }
    if (kCLanes == 2) {
      ax += __shfl_xor_sync(0xffffffffu, ax, 1);
      ay += __shfl_xor_sync(0xffffffffu, ay, 1);
      az += __shfl_xor_sync(0xffffffffu, az, 1);
    }
    fx = ax;
    fy = ay;
    fz = az;
    if (helpers) {  // partial sums of helper slots, in order
      if (lane == 0 && valid) {
        part[3 * q] = fx;
        part[3 * q + 1] = fy;
        part[3 * q + 2] = fz;
      }
      __syncthreads();
      if (primary && lane == 0)
        for (int k = 1; k <= nh; ++k) {
          fx += part[3 * (q + k)];
          fy += part[3 * (q + k) + 1];
          fz += part[3 * (q + k) + 2];
        }
    }
    if (hub_local >= 0) {  // the hub's force: negated partner forces, summed over the tile
      __shared__ float red[3 * 32];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        rx += __shfl_xor_sync(0xffffffffu, rx, o);
        ry += __shfl_xor_sync(0xffffffffu, ry, o);
        rz += __shfl_xor_sync(0xffffffffu, rz, o);
      }
      const int wid = threadIdx.x >> 5;
      if ((threadIdx.x & 31) == 0) {
        red[3 * wid] = rx;
        red[3 * wid + 1] = ry;
        red[3 * wid + 2] = rz;
      }
      __syncthreads();
      if (q == hub_local && lane == 0) {
        const int nw = (int)((blockDim.x + 31) >> 5);
        for (int w = 0; w < nw; ++w) {
          fx += red[3 * w];
          fy += red[3 * w + 1];
          fz += red[3 * w + 2];
        }
      }
      __syncthreads();
    }
  };
  // v += F kick; x += v dt with x kept as an unevaluated float sum hi + lo
  auto advance = [&](float kick) {
    if (moves && lane == 0) {
      const float f[3] = {fx, fy, fz};
      for (int d = 0; d < 3; ++d) {
        v[d] = fmaf(f[d], kick, v[d]);
        // TwoSum (Knuth) then Fast2Sum; the _rn intrinsics keep every rounding explicit
        const float dx = __fmul_rn(v[d], fdt);
        const float sum = __fadd_rn(xh[d], dx);
        const float bv = __fsub_rn(sum, xh[d]);
        const float err = __fadd_rn(__fsub_rn(xh[d], __fsub_rn(sum, bv)), __fsub_rn(dx, bv));
        const float lo = __fadd_rn(xl[d], err);
        xh[d] = __fadd_rn(sum, lo);
        xl[d] = __fsub_rn(lo, __fsub_rn(xh[d], sum));
      }
    }
    if (nbuf == 1) cluster.sync();  // one buffer: every read of this substep is done
    if (primary && lane == 0) buf(cur ^ 1).put(q, xh, xl);
    cluster.sync();
    cur ^= 1;
  };

  evaluate();
  advance(0.5f * fdt);  // md_loop_start
  evaluate();
  for (int k = 1; k < a.n; ++k) {  // md_loop
    advance(fdt);
    evaluate();
  }
  const double t = a.t_end;
  if (moves && lane == 0) {  // md_loop_stop
    v[0] = fmaf(fx, 0.5f * fdt, v[0]);
    v[1] = fmaf(fy, 0.5f * fdt, v[1]);
    v[2] = fmaf(fz, 0.5f * fdt, v[2]);
  }
  if (primary && lane == 0) {
    const double x = (double)xh[0] + (double)xl[0], y = (double)xh[1] + (double)xl[1],
                 z = (double)xh[2] + (double)xl[2];
    m.x[0][slot] = x;
    m.y[0][slot] = y;
    m.z[0][slot] = z;
    m.vx[slot] = v[0];
    m.vy[slot] = v[1];
    m.vz[slot] = v[2];
    if (moves) bin(x, y, z, (double)v[0], (double)v[1], (double)v[2]);
  }
  for (int k = threadIdx.x; k < nbond; k += blockDim.x) {
    m.newlen[bond0 + k] = (double)bnew[k];
    m.oldlen[bond0 + k] = (double)bold[k];
    m.diag[bond0 + k] = (double)bdiag[k];
  }
  // switch_logic (src/cilia.cpp:241-258, src/ConstantBeatCilia.cpp:8-23)
  for (int c = c0 + (int)threadIdx.x; c < c1; c += (int)blockDim.x) {
    const CiliumDev cl = m.cil[c];
    double mp = m.midpnt[c], ts = m.tstroke[c];
    if (cl.kind == 1) {
      if (t - ts >= cl.power_dur && mp == cl.start) mp += 1;
      if (t - ts - cl.power_dur >= cl.recovery_dur && mp > cl.start) {
        ts = t;
        mp = cl.start;
      }
    } else {
      if (mp == cl.start && t - ts > 100.0) mp += 1;
      const int l0 = cl.slot0 - base;
      double lb = 0.0;
      const PBuf B = buf(cur);
      const int sd = cl.stride;
      for (int i = 0; i < cl.len - 1; ++i)
        lb += 2.0f * B.dist(l0 + sd * i, l0 + sd * (i + 1)) -
              B.dist(l0 + sd * (cl.len + i), l0 + sd * (cl.len + i + 1)) -
              B.dist(l0 + sd * (2 * cl.len + i), l0 + sd * (2 * cl.len + i + 1));
      if (lb > (float)cl.max_bend && mp > cl.start) {
        ts = t;
        mp = cl.start;
      }
    }
    if (mp > cl.start) mp += a.tstep / cl.m_speed;
    m.midpnt[c] = mp;
    m.tstroke[c] = ts;
  }
  cluster.sync();  // no CTA leaves while another may still read its shared memory
}

template <int kCLanes, typename Bin>
__global__ void __launch_bounds__(1024, 1) k_md_cluster(MDState m, MDStepArgs a, Bin bin, ClusterLayout lay) {
  md_cluster_body<kCLanes>(m, a, bin, lay, (int)blockIdx.x);
}

struct ClBinF64 {
  static constexpr bool kCollide = false;
  __device__ double collide(const double*, float*) const { return 0.0; }
  __device__ void add_diss(double) const {}
  CellsF64 c;
  Box box;
  double an[3];
  double mb;
  unsigned* err;
  __device__ void operator()(double x, double y, double z, double vx, double vy, double vz) const {
    const long cid = unwrapped_cell(box, an, x, y, z);
    if (cid < 0) {
      atomicOr(err, kErrCellRange);
      return;
    }
    double* sp = reinterpret_cast<double*>(c.sum + cid);
    atomicAdd(sp + 0, vx * mb);
    atomicAdd(sp + 1, vy * mb);
    atomicAdd(sp + 2, vz * mb);
    atomicAdd(sp + 3, mb * (vx * vx + vy * vy + vz * vz));
    atomicAdd(c.cnt + cid, 1u << 16);
  }
};

struct ClBinF32 {
  static constexpr bool kCollide = false;
  __device__ double collide(const double*, float*) const { return 0.0; }
  __device__ void add_diss(double) const {}
  CellsF32 c;
  Box box;
  double an[3];
  float mb;
  unsigned* err;
  __device__ void operator()(double x, double y, double z, double vx, double vy, double vz) const {
    const long cid = unwrapped_cell(box, an, x, y, z);
    if (cid < 0) {
      atomicOr(err, kErrCellRange);
      return;
    }
    const float fvx = (float)vx, fvy = (float)vy, fvz = (float)vz;
    float* sp = reinterpret_cast<float*>(c.sum + cid);
    atomicAdd(sp + 0, fvx * mb);
    atomicAdd(sp + 1, fvy * mb);
    atomicAdd(sp + 2, fvz * mb);
    atomicAdd(sp + 3, mb * (fvx * fvx + fvy * fvy + fvz * fvz));
    atomicAdd(c.cnt + cid, 1u << 16);
  }
};

// Binning and bead collision of one replica of a batch (cells of the arena,
// offset by the replica's first cell).  The fields live in shared memory and
// are read only at the start and end of the launch, so they hold no
// registers through the substeps.
struct BatchBinData {
  float4* sum;
  uint32_t* cnt;
  const float4* par;
  long cell0;
  Box box;
  double a_cur[3], a_next[3];
  float mb;
  double mbd;
  unsigned* err;
  double* diss;
};

struct BatchBin {
  static constexpr bool kCollide = true;
  const BatchBinData* d;
  // MDObject beads in the collision (MPCD::next_tstep, src/libcilia/mpcd.cpp:140-247)
  __device__ double collide(const double* X, float* v) const {
    const long cid = unwrapped_cell(d->box, d->a_cur, X[0], X[1], X[2]);
    if (cid < 0) {
      atomicOr(d->err, kErrCellRange);
      return 0.0;
    }
    apply_map_f32(d->par + 2 * (d->cell0 + cid), v[0], v[1], v[2]);
    return d->mbd * ((double)v[0] * v[0] + (double)v[1] * v[1] + (double)v[2] * v[2]);
  }
  __device__ void add_diss(double x) const { atomicAdd(d->diss, x); }
  // md_loop_stop's binning with the next shift (src/libcilia/mdobject.cpp:62-72)
  __device__ void operator()(double x, double y, double z, double vx, double vy, double vz) const {
    const long cid = unwrapped_cell(d->box, d->a_next, x, y, z);
    if (cid < 0) {
      atomicOr(d->err, kErrCellRange);
      return;
    }
    const float mb = d->mb;
    const float fvx = (float)vx, fvy = (float)vy, fvz = (float)vz;
    red_add_v4(d->sum + d->cell0 + cid,
               make_float4(fvx * mb, fvy * mb, fvz * mb, mb * (fvx * fvx + fvy * fvy + fvz * fvz)));
    atomicAdd(d->cnt + d->cell0 + cid, 1u << 16);
  }
};

// One cluster of `ctiles` CTAs per listed replica; inactive replicas leave at
// once (the whole cluster together).
template <int kCLanes>
__global__ void __launch_bounds__(1024, 1)
    k_md_cluster_batch(MDState m, BatchTables t, BatchCells c, const int* reps, int ctiles, ClusterLayout lay) {
  __shared__ MDStepArgs sa;
  __shared__ BatchBinData sb;
  const int r = reps[blockIdx.x / ctiles];
  if (!t.step[r].active) return;
  const BatchRep& R = t.rep[r];
  if (threadIdx.x == 0) {
    sa = t.step[r].md;
    sb.sum = c.sum;
    sb.cnt = c.cnt;
    sb.par = c.par;
    sb.cell0 = R.cell0;
    sb.box = sa.box;
    for (int q = 0; q < 3; ++q) {
      sb.a_cur[q] = sa.a_cur[q];
      sb.a_next[q] = sa.a_next[q];
    }
    sb.mb = (float)R.bead_mass;
    sb.mbd = R.bead_mass;
    sb.err = &t.state[r].err;
    sb.diss = &t.state[r].diss;
  }
  __syncthreads();
  const BatchBin bin{&sb};
  md_cluster_body<kCLanes>(m, sa, bin, lay, R.md_tile0 + (int)(blockIdx.x % ctiles));
}

template <int L, typename Bin>
cudaError_t launch_cluster_l(const MDState& m, const MDStepArgs& a, const Bin& bin, cudaStream_t s) {
  ClusterLayout lay{cl_np(m.tile, m.hmax), m.cl_nsp_max, m.cl_nbond_max, m.cl_nbuf};
  const size_t smem = lay.bytes(m.tile);
  auto kern = k_md_cluster<L, Bin>;
  cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(m.ntiles);
  cfg.blockDim = dim3(L * m.tile);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = m.ntiles;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, m, a, bin, lay);
}

template <typename Bin>
cudaError_t launch_cluster(const MDState& m, const MDStepArgs& a, const Bin& bin, cudaStream_t s) {
  return m.cl_lanes == 2 ? launch_cluster_l<2>(m, a, bin, s) : launch_cluster_l<1>(m, a, bin, s);
}

}  // namespace

size_t md_cluster_smem(const MDState& m) {
  ClusterLayout lay{cl_np(m.tile, m.hmax), m.cl_nsp_max, m.cl_nbond_max, m.cl_nbuf};
  return lay.bytes(m.tile);
}

// 1 when a cluster of m.ntiles CTAs with this layout can be scheduled
template <int L>
int cluster_feasible_l(const MDState& m) {
  if (m.ntiles < 1 || m.ntiles > 16 || L * m.tile > 1024) return 0;
  const size_t smem = md_cluster_smem(m);
  if (smem > 227 * 1024) return 0;
  auto kern = k_md_cluster<L, ClBinF32>;
  cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(m.ntiles);
  cfg.blockDim = dim3(L * m.tile);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = m.ntiles;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int nclusters = 0;
  if (cudaOccupancyMaxActiveClusters(&nclusters, (const void*)kern, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return nclusters >= 1;
}

int md_cluster_feasible(const MDState& m) {
  return m.cl_lanes == 2 ? cluster_feasible_l<2>(m) : cluster_feasible_l<1>(m);
}

size_t md_cluster_batch_smem(int tile, int hmax, int nsp_max, int nbond_max, int nbuf) {
  ClusterLayout lay{cl_np(tile, hmax), nsp_max, nbond_max, nbuf};
  return lay.bytes(tile);
}

namespace {
template <int L>
cudaLaunchConfig_t batch_cfg(int nclusters, int tile, int ctiles, size_t smem, cudaStream_t s,
                             cudaLaunchAttribute* attr) {
  auto kern = k_md_cluster_batch<L>;
  cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nclusters * ctiles);
  cfg.blockDim = dim3(L * tile);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = ctiles;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}
}  // namespace

int md_cluster_batch_feasible(int lanes, int tile, int ctiles, size_t smem) {
  if (ctiles < 1 || ctiles > kMaxClusterTiles || lanes * tile > 1024 || smem + sizeof(MDStepArgs) > 227 * 1024) return 0;
  cudaLaunchAttribute attr[1];
  int n = 0;
  cudaError_t e;
  if (lanes == 2) {
    cudaLaunchConfig_t cfg = batch_cfg<2>(1, tile, ctiles, smem, nullptr, attr);
    e = cudaOccupancyMaxActiveClusters(&n, (const void*)k_md_cluster_batch<2>, &cfg);
  } else {
    cudaLaunchConfig_t cfg = batch_cfg<1>(1, tile, ctiles, smem, nullptr, attr);
    e = cudaOccupancyMaxActiveClusters(&n, (const void*)k_md_cluster_batch<1>, &cfg);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n >= 1;
}

int launch_md_cluster_batch(const MDState& m, const BatchTables& t, BatchCells c, const int* reps, int nreps,
                            int ctiles, int hmax, int nsp_max, int nbond_max, int nbuf, cudaStream_t s,
                            cudaError_t* st) {
  if (nreps <= 0) return 0;
  ClusterLayout lay{cl_np(m.tile, hmax), nsp_max, nbond_max, nbuf};
  const size_t smem = lay.bytes(m.tile);
  cudaLaunchAttribute attr[1];
  if (m.cl_lanes == 2) {
    cudaLaunchConfig_t cfg = batch_cfg<2>(nreps, m.tile, ctiles, smem, s, attr);
    *st = cudaLaunchKernelEx(&cfg, k_md_cluster_batch<2>, m, t, c, reps, ctiles, lay);
  } else {
    cudaLaunchConfig_t cfg = batch_cfg<1>(nreps, m.tile, ctiles, smem, s, attr);
    *st = cudaLaunchKernelEx(&cfg, k_md_cluster_batch<1>, m, t, c, reps, ctiles, lay);
  }
  return 1;
}

int launch_md_cluster_f64cells(const MDState& m, const CellsF64& c, const MDStepArgs& a, cudaStream_t s,
                               cudaError_t* st) {
  if (m.nslots == 0) return 0;
  ClBinF64 bin{c, a.box, {a.a_next[0], a.a_next[1], a.a_next[2]}, a.bead_mass, a.err};
  *st = launch_cluster(m, a, bin, s);
  return 1;
}

int launch_md_cluster_f32cells(const MDState& m, const CellsF32& c, const MDStepArgs& a, cudaStream_t s,
                               cudaError_t* st) {
  if (m.nslots == 0) return 0;
  ClBinF32 bin{c, a.box, {a.a_next[0], a.a_next[1], a.a_next[2]}, (float)a.bead_mass, a.err};
  *st = launch_cluster(m, a, bin, s);
  return 1;
}

}  // namespace mpcd
