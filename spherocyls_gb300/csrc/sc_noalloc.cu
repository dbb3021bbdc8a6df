// sc_noalloc.cu -- sc_forces_noalloc: contact forces of one box from caller-owned
// device arrays, with no device or host allocation by the library.
//
// Some callers cannot let a library allocate device memory: a host program that
// has already divided the GPU's memory among its own solvers and hands out only
// pre-allocated buffers, or a real-time loop that must never hit the allocator.
// For them this entry point computes the same forces as sc_calc_forces on an FP64
// handle (the reference's calc_forces, tmarschall/spherocyls
// src/cpp/strain_dynamics.cpp:137-153) but keeps its cell lists in one file-scope
// __device__ array of fixed size instead of memory from cudaMalloc.
//
// The scratch array exists once per GPU that loads the library and stays resident
// until the process exits.  Its device address is looked up once per device
// (cudaGetSymbolAddress, with that device current) on the first call made on that
// device and kept for the process; make that first call before any stream capture,
// and make no call on a device after cudaDeviceReset on it (the reset unloads the
// module, so the kept address no longer names the array).  Every call shares the
// array and leaves the previous call's lists in it; the cell counters are cleared
// at the start of each call.  Calls whose work overlaps on the GPU (two streams,
// or two host threads on one device) race on the array: serialise them.
//
// Compiled with -fmad=false, like the FP64 force pass, so each pair contribution
// uses the reference's operation order.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "../../include/spherocyl.h"
#include "sc_internal.hpp"
#include "sc_pair.cuh"

namespace sc {
namespace {

constexpr int kNaMaxN = SC_NOALLOC_MAX_PARTICLES;
constexpr int kNaMaxCells = 16384;  // finer grids are coarsened: larger cells stay correct
constexpr int kNaHeader = 64;       // ints: grid parameters (doubles at even offsets)
constexpr int kNaInts = kNaHeader + 2 * kNaMaxCells + 3 * kNaMaxN;

// The only scratch the entry point uses (about 0.9 MB per device).
static __device__ __align__(256) int g_na_scratch[kNaInts];

struct NaView {
  double* hdr_d;  // [0] W, [1] H, [2] pad used for the grid, [3] Rmax+Amax
  int* hdr_i;     // [8] cols, [9] rows
  int* count;
  int* start;
  int* cell_of;
  int* rank;
  int* sorted;
};

__host__ __device__ inline NaView na_view(int* base) {
  NaView v;
  v.hdr_d = reinterpret_cast<double*>(base);
  v.hdr_i = base;
  v.count = base + kNaHeader;
  v.start = v.count + kNaMaxCells;
  v.cell_of = v.start + kNaMaxCells;
  v.rank = v.cell_of + kNaMaxN;
  v.sorted = v.rank + kNaMaxN;
  return v;
}

// configure_cells (src/cpp/spherocyl_box.cpp:223-241) on the device: the largest
// R and A, the grid, and a cleared counter for every cell used.  The cell width
// factor is the reference's 2.24 for |gamma| <= 1/2 and 2 sqrt(1 + gamma^2) beyond
// (the width the handle's grid takes for shear past gamma = 1/2): in sheared
// coordinates two touching spines are at most 2 (R + A) sqrt(1 + gamma^2) apart in
// x, so the 3x3 block of cells holds every contact at any gamma.
__global__ void k_na_setup(int* scratch, int n, double L, double pad, double wfac,
                           const double* R, const double* A) {
  NaView v = na_view(scratch);
  __shared__ double sr[256], sa[256];
  double r = 0.0, a = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    r = fmax(r, R[i]);
    a = fmax(a, A[i]);
  }
  sr[threadIdx.x] = r;
  sa[threadIdx.x] = a;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sr[threadIdx.x] = fmax(sr[threadIdx.x], sr[threadIdx.x + o]);
      sa[threadIdx.x] = fmax(sa[threadIdx.x], sa[threadIdx.x + o]);
    }
    __syncthreads();
  }
  __shared__ int dims[2];
  if (threadIdx.x == 0) {
    double ra = sr[0] + sa[0];
    double wmin = wfac * ra + pad, hmin = 2 * ra + pad;
    int rows = (int)(L / hmin), cols = (int)(L / wmin);
    rows = rows > 1 ? rows : 1;
    cols = cols > 1 ? cols : 1;
    while ((long long)rows * cols > kNaMaxCells) {  // coarsen: fewer, larger cells
      rows = rows > 1 ? (rows + 1) / 2 : 1;
      cols = cols > 1 ? (cols + 1) / 2 : 1;
    }
    v.hdr_d[0] = L / cols;
    v.hdr_d[1] = L / rows;
    v.hdr_d[2] = pad;
    v.hdr_d[3] = ra;
    v.hdr_i[8] = cols;
    v.hdr_i[9] = rows;
    dims[0] = cols;
    dims[1] = rows;
  }
  __syncthreads();
  int nc = dims[0] * dims[1];
  for (int c = threadIdx.x; c < nc; c += blockDim.x) v.count[c] = 0;
}

__device__ __forceinline__ double na_wrap(double v, double L) {
  // the reference's wrap loops, bounded; a runaway value is clamped onto the grid
  for (int it = 0; it < 64 && v > L; it++) v -= L;
  for (int it = 0; it < 64 && v < 0.0; it++) v += L;
  return v;
}

__global__ void k_na_hash(int* scratch, int n, double L, const double* x, const double* y) {
  NaView v = na_view(scratch);
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int cols = v.hdr_i[8], rows = v.hdr_i[9];
  double px = na_wrap(x[i], L), py = na_wrap(y[i], L);
  int col = (int)(px / v.hdr_d[0]), rw = (int)(py / v.hdr_d[1]);
  col = col < 0 ? 0 : (col >= cols ? cols - 1 : col);
  rw = rw < 0 ? 0 : (rw >= rows ? rows - 1 : rw);
  int c = col + rw * cols;
  v.cell_of[i] = c;
  v.rank[i] = atomicAdd(&v.count[c], 1);
}

// exclusive scan of the cell counts in one 1024-thread block
__global__ void __launch_bounds__(1024) k_na_scan(int* scratch) {
  NaView v = na_view(scratch);
  const int nc = v.hdr_i[8] * v.hdr_i[9];
  __shared__ int warp_tot[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int base = 0; base < nc; base += 1024) {
    int k = base + threadIdx.x;
    int val = k < nc ? v.count[k] : 0;
    int xs = val;
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, xs, o);
      if (lane >= o) xs += t;
    }
    if (lane == 31) warp_tot[w] = xs;
    __syncthreads();
    if (w == 0) {
      int t = warp_tot[lane];
      for (int o = 1; o < 32; o <<= 1) {
        int u = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += u;
      }
      warp_tot[lane] = t;
    }
    __syncthreads();
    int excl = xs - val + (w > 0 ? warp_tot[w - 1] : 0) + carry;
    if (k < nc) v.start[k] = excl;
    __syncthreads();
    if (threadIdx.x == 1023) carry = excl + val;
    __syncthreads();
  }
}

__global__ void k_na_scatter(int* scratch, int n) {
  NaView v = na_view(scratch);
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  v.sorted[v.start[v.cell_of[i]] + v.rank[i]] = i;
}

// particle order inside each cell, so repeated calls sum in the same order
__global__ void k_na_cellsort(int* scratch) {
  NaView v = na_view(scratch);
  const int nc = v.hdr_i[8] * v.hdr_i[9];
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  int* P = v.sorted + v.start[c];
  int m = v.count[c];
  for (int k = 1; k < m; k++) {
    int key = P[k], j = k - 1;
    while (j >= 0 && P[j] > key) {
      P[j + 1] = P[j];
      j--;
    }
    P[j + 1] = key;
  }
}

// Every overlapping pair among the 3x3 block of cells (each distinct cell once),
// computed with the lower particle index as the reference's "p".
__global__ void __launch_bounds__(128) k_na_forces(int* scratch, int n, double L, double gamma,
                                                  const double* x, const double* y,
                                                  const double* phi, const double* R,
                                                  const double* A, double* fx, double* fy,
                                                  double* tau) {
  NaView v = na_view(scratch);
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int cols = v.hdr_i[8], rows = v.hdr_i[9];
  const int c = v.cell_of[i];
  const int col = c % cols, rw = c / cols;
  const int ncx = cols < 3 ? cols : 3, ncy = rows < 3 ? rows : 3;
  double xi = x[i], yi = y[i], Ai = A[i], Ri = R[i];
  double nxi = Ai * cos(phi[i]), nyi = Ai * sin(phi[i]);
  double Fx = 0.0, Fy = 0.0, T = 0.0;
  for (int a = 0; a < ncy; a++) {
    int r2 = ncy == 3 ? wrap_index(rw + a - 1, rows) : a;
    for (int b = 0; b < ncx; b++) {
      int c2 = ncx == 3 ? wrap_index(col + b - 1, cols) : b;
      int cc = c2 + r2 * cols;
      int st = v.start[cc], en = st + v.count[cc];
      for (int k = st; k < en; k++) {
        int j = v.sorted[k];
        if (j == i) continue;
        double Aj = A[j];
        double nxj = Aj * cos(phi[j]), nyj = Aj * sin(phi[j]);
        PairF64 o;
        if (i < j) {
          if (pair_fp64<false>(xi - x[j], yi - y[j], nxi, nyi, Ai, nxj, nyj, Aj, Ri + R[j], gamma,
                               L, L, false, 2.0, o)) {
            Fx += o.fx;
            Fy += o.fy;
            T += o.tp;
          }
        } else {
          if (pair_fp64<false>(x[j] - xi, y[j] - yi, nxj, nyj, Aj, nxi, nyi, Ai, R[j] + Ri, gamma,
                               L, L, false, 2.0, o)) {
            Fx -= o.fx;
            Fy -= o.fy;
            T += o.tq;
          }
        }
      }
    }
  }
  fx[i] = Fx;
  fy[i] = Fy;
  tau[i] = T;
}

std::mutex g_na_mutex;
int* g_na_addr[64] = {nullptr};
thread_local std::string g_na_error;

}  // namespace
}  // namespace sc

extern "C" const char* sc_noalloc_last_error(void) { return sc::g_na_error.c_str(); }

extern "C" int sc_forces_noalloc(int n, double L, double gamma, double pad, const double* x,
                                 const double* y, const double* phi, const double* R,
                                 const double* A, double* fx, double* fy, double* tau,
                                 void* stream) {
  using namespace sc;
  g_na_error.clear();
  if (n < 2 || n > kNaMaxN) {
    g_na_error = "sc_forces_noalloc: n must be in [2, " + std::to_string(kNaMaxN) +
                 "] (the fixed scratch holds at most that many particles)";
    return SC_E_ARG;
  }
  if (!(L > 0) || !(pad >= 0) || !x || !y || !phi || !R || !A || !fx || !fy || !tau) {
    g_na_error = "sc_forces_noalloc: L > 0, pad >= 0 and all ten device arrays are required";
    return SC_E_ARG;
  }
  if (!std::isfinite(gamma) || std::fabs(gamma) > 1e6) {
    g_na_error = "sc_forces_noalloc: gamma must be finite (|gamma| <= 1e6)";
    return SC_E_ARG;
  }
  // the sheared-grid width factor of the handle's grid (see k_na_setup)
  const double wfac = std::fabs(gamma) > 0.5 ? 2 * std::sqrt(gamma * gamma + 1) : 2.24;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    g_na_error = "sc_forces_noalloc: no current CUDA device";
    return SC_E_CUDA;
  }
  int* scratch = nullptr;
  {
    // one-time set-up per device, with that device current
    std::lock_guard<std::mutex> lk(g_na_mutex);
    if (!g_na_addr[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_na_scratch);
      if (e != cudaSuccess || !p) {
        g_na_error = std::string("sc_forces_noalloc: cudaGetSymbolAddress: ") +
                     cudaGetErrorString(e);
        return SC_E_CUDA;
      }
      g_na_addr[dev] = static_cast<int*>(p);
    }
    scratch = g_na_addr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_na_setup<<<1, 256, 0, st>>>(scratch, n, L, pad, wfac, R, A);
  int grid = (n + 255) / 256;
  k_na_hash<<<grid, 256, 0, st>>>(scratch, n, L, x, y);
  k_na_scan<<<1, 1024, 0, st>>>(scratch);
  k_na_scatter<<<grid, 256, 0, st>>>(scratch, n);
  k_na_cellsort<<<(kNaMaxCells + 127) / 128, 128, 0, st>>>(scratch);
  k_na_forces<<<(n + 127) / 128, 128, 0, st>>>(scratch, n, L, gamma, x, y, phi, R, A, fx, fy,
                                                tau);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_na_error = std::string("sc_forces_noalloc: launch: ") + cudaGetErrorString(e);
    return SC_E_CUDA;
  }
  return SC_OK;
}
