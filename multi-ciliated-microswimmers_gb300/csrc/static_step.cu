// mpcd_fluid_step_noalloc: one split-precision MPC step of a plain fluid on
// caller-owned device arrays, for callers that cannot allocate device memory
// themselves (code running inside another runtime's memory pool or allocator,
// or plug-ins that are only handed pointers and a stream).  It calls no
// cudaMalloc, cudaFree or allocating library routine.
//
// Its per-cell scratch (velocity sums, counts and collision maps) lives in one
// file-scope static device array sized for kMaxCells cells.  Every GPU that
// loads the library holds that array until the process exits; every call
// shares it, so calls that overlap on the GPU (different streams or threads)
// race, and the array keeps the last call's contents (the sums are cleared at
// the start of each call).  Particles that break the layout (a cell index
// beyond the box, an offset outside [0,1)) are rejected before any kernel
// touches the scratch.
#include <algorithm>
#include <cstring>
#include <mutex>

#include "../../include/mpcd_gpu.h"
#include "engine_internal.h"

using namespace mpcd;

namespace {

constexpr long kMaxCells = MPCD_NOALLOC_MAX_CELLS;
// layout: sums (float4 per cell) | maps (2 float4 per cell) | counts (uint32 per cell)
//         | dissipated energy (double) | error word (unsigned)
constexpr size_t kSumBytes = sizeof(float4) * kMaxCells;
constexpr size_t kParBytes = 2 * sizeof(float4) * kMaxCells;
constexpr size_t kCntBytes = sizeof(uint32_t) * kMaxCells;
constexpr size_t kScratchBytes = kSumBytes + kParBytes + kCntBytes + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct DeviceScratch {
  bool ready = false;
  unsigned char* base = nullptr;  // device address of g_noalloc_scratch
};

std::mutex g_setup_mutex;
DeviceScratch g_scratch[64];

// Resolves the array's device address on the current device, once per device.
cudaError_t scratch_for_device(int dev, unsigned char** out) {
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch[dev].ready) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch[dev].base = static_cast<unsigned char*>(p);
    g_scratch[dev].ready = true;
  }
  *out = g_scratch[dev].base;
  return cudaSuccess;
}

// Caller-packed particles are checked before any kernel indexes the scratch
// with them: every axis' cell index below the box edge and every offset in
// [0,1) (NaN fails).  A bad particle sets kErrCellRange in *err.
__global__ void k_check_split_f32(FluidF32 f, Box box, unsigned* err) {
  unsigned bad = 0;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < f.n; i += (long)gridDim.x * blockDim.x) {
    const float4 p = f.pos[i];
    const uint32_t cp = __float_as_uint(p.w);
    const bool ok = (cp >> 30) == 0u && cell_x(cp) < box.L[0] && cell_y(cp) < box.L[1] && cell_z(cp) < box.L[2] &&
                    p.x >= 0.0f && p.x < 1.0f && p.y >= 0.0f && p.y < 1.0f && p.z >= 0.0f && p.z < 1.0f;
    if (!ok) bad = 1u;
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(err, kErrCellRange);
}

}  // namespace

extern "C" int mpcd_fluid_step_noalloc(const int* sizes, long n, void* pos, void* vel, double tstep,
                                       const double* a_cur, const double* a_next, unsigned long long seed,
                                       unsigned long long step, double* diss, void* stream) {
  if (!sizes || !a_cur || !a_next || n < 0 || (n > 0 && (!pos || !vel)) || !(tstep > 0)) return MPCD_EINVAL;
  long ncell = 1;
  for (int q = 0; q < 3; ++q) {
    if (sizes[q] < 2 || sizes[q] > 1024) return MPCD_EINVAL;
    ncell *= sizes[q];
  }
  if (ncell > kMaxCells) return MPCD_EINVAL;  // the box exceeds the static scratch
  for (int q = 0; q < 3; ++q)
    if (!(a_cur[q] >= 0.0 && a_cur[q] < 1.0) || !(a_next[q] >= 0.0 && a_next[q] < 1.0)) return MPCD_EINVAL;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return MPCD_ECUDA;
  unsigned char* base = nullptr;
  if (scratch_for_device(dev, &base) != cudaSuccess) return MPCD_ECUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  CellsF32 cells;
  cells.ncell = ncell;
  cells.sum = reinterpret_cast<float4*>(base);
  cells.par = reinterpret_cast<float4*>(base + kSumBytes);
  cells.cnt = reinterpret_cast<uint32_t*>(base + kSumBytes + kParBytes);
  double* d_diss = reinterpret_cast<double*>(base + kSumBytes + kParBytes + kCntBytes);
  unsigned* d_err = reinterpret_cast<unsigned*>(d_diss + 1);
  FluidF32 f;
  f.n = n;
  f.pos = static_cast<float4*>(pos);
  f.vel = static_cast<float4*>(vel);
  // clear what must start at zero: the sums, counts, energy and error word
  if (cudaMemsetAsync(cells.sum, 0, sizeof(float4) * ncell, s) != cudaSuccess) return MPCD_ECUDA;
  if (cudaMemsetAsync(cells.cnt, 0, sizeof(uint32_t) * ncell, s) != cudaSuccess) return MPCD_ECUDA;
  if (cudaMemsetAsync(d_diss, 0, sizeof(double) + sizeof(unsigned), s) != cudaSuccess) return MPCD_ECUDA;
  unsigned err_h = 0;
  if (n > 0) {
    // the caller's layout is checked first: a cell index beyond the box would
    // send the binning's atomics past the scratch array
    Box box{{sizes[0], sizes[1], sizes[2]}};
    const long g = std::min<long>((n + 255) / 256, 4096);
    k_check_split_f32<<<(int)g, 256, 0, s>>>(f, box, d_err);
    if (cudaGetLastError() != cudaSuccess) return MPCD_ECUDA;
    if (cudaMemcpyAsync(&err_h, d_err, sizeof err_h, cudaMemcpyDeviceToHost, s) != cudaSuccess) return MPCD_ECUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return MPCD_ECUDA;
    if (err_h) return MPCD_EDEVICE;  // nothing was changed
  }
  StepArgs a{};
  for (int q = 0; q < 3; ++q) {
    a.box.L[q] = sizes[q];
    a.a_cur[q] = a_cur[q];
    a.a_next[q] = a_next[q];
    a.ta_cur[q] = 1.0 - a_cur[q];
    a.ta_next[q] = 1.0 - a_next[q];
    a.fta_cur[q] = (float)a.ta_cur[q];
    a.fta_next[q] = (float)a.ta_next[q];
  }
  a.h = tstep;
  a.fh = (float)tstep;
  a.bead_mass = 5.0;
  a.fbead_mass = 5.0f;
  a.seed = seed;
  a.step = step;
  a.err = d_err;
  a.diss = d_diss;
  launch_bin_fluid_f32(f, cells, a, s);     // sums with the current shift
  launch_cell_params_f32(cells, a, s);      // collision maps (clears the sums)
  launch_fluid_step_f32(f, cells, a, s);    // collide, stream, bin with the next shift
  if (cudaGetLastError() != cudaSuccess) return MPCD_ECUDA;
  double diss_h = 0.0;
  if (cudaMemcpyAsync(&diss_h, d_diss, sizeof diss_h, cudaMemcpyDeviceToHost, s) != cudaSuccess) return MPCD_ECUDA;
  if (cudaMemcpyAsync(&err_h, d_err, sizeof err_h, cudaMemcpyDeviceToHost, s) != cudaSuccess) return MPCD_ECUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return MPCD_ECUDA;
  if (diss) *diss = diss_h;
  return err_h ? MPCD_EDEVICE : MPCD_OK;
}
