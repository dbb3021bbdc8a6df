// sc_gen_device.cu -- crossing-free random packings generated on the GPU.
//
// The reference places particles one after another, redrawing each until it has
// no contact or crossing with those already placed (random_configuration and
// check_particle_cross, src/cpp/spherocyl_box.cpp:597-790; place_spherocyls,
// src/cuda/spherocyl_box.cpp:1063-1200), and sc_generate_packing does the same on
// the host.  For large N the placement here runs in rounds on the device: every
// particle still to place draws a position and angle from a counter-based hash of
// (seed, particle, round), the particles are binned into cells at least one
// interaction reach wide, and a particle is redrawn in the next round when its spine
// comes closer than min_sep (R_i + R_j) to that of any lower-numbered particle.
// Particles below the lowest one redrawn in a round never move again, so the
// placed prefix only grows and the rounds end; the result depends only on the seed
// (no atomics decide anything), not on the schedule.  The packing fraction, box
// and shapes are those of sc_generate_packing; the random sequence is not.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/spherocyl.h"
#include "sc_segments.hpp"

namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// uniform in [0, 1) from (seed, particle, round, component)
__device__ __forceinline__ double hash_u01(uint64_t seed, uint64_t i, uint64_t round, int k) {
  uint64_t h = mix64(seed ^ mix64(i * 0xD1B54A32D192ED03ull + round));
  h = mix64(h + (uint64_t)k * 0x9E3779B97F4A7C15ull);
  return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

struct Gen {
  int n, ng;
  double L, gw, sep, a_over_r, r_small, r_ratio;
  uint64_t seed;
  double *x, *y, *phi;
  int *cell, *rank, *count, *start, *list, *redraw, *nredraw;
};

__device__ __forceinline__ double radius(const Gen& g, int i) {
  return (i % 2 == 0) ? g.r_small : g.r_small * g.r_ratio;
}

__global__ void k_draw(Gen g, int round) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n || !g.redraw[i]) return;
  const double pi = 3.14159265358979323846;
  g.x[i] = g.L * hash_u01(g.seed, i, round, 0);
  g.y[i] = g.L * hash_u01(g.seed, i, round, 1);
  g.phi[i] = pi * hash_u01(g.seed, i, round, 2);
}

__global__ void k_bin(Gen g) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  int cx = (int)(g.x[i] / g.gw), cy = (int)(g.y[i] / g.gw);
  cx = cx < 0 ? 0 : (cx >= g.ng ? g.ng - 1 : cx);
  cy = cy < 0 ? 0 : (cy >= g.ng ? g.ng - 1 : cy);
  const int c = cy * g.ng + cx;
  g.cell[i] = c;
  g.rank[i] = atomicAdd(&g.count[c], 1);
}

// exclusive scan of the cell counts, one block
__global__ void __launch_bounds__(1024) k_scan(Gen g) {
  __shared__ int sh[1024];
  const int nc = g.ng * g.ng;
  const int per = (nc + blockDim.x - 1) / blockDim.x;
  const int b = threadIdx.x * per, e = b + per < nc ? b + per : nc;
  int sum = 0;
  for (int c = b; c < e; c++) sum += g.count[c];
  sh[threadIdx.x] = sum;
  __syncthreads();
  for (int o = 1; o < (int)blockDim.x; o <<= 1) {
    const int v = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += v;
    __syncthreads();
  }
  int run = sh[threadIdx.x] - sum;
  for (int c = b; c < e; c++) {
    g.start[c] = run;
    run += g.count[c];
  }
}

__global__ void k_fill(Gen g) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  g.list[g.start[g.cell[i]] + g.rank[i]] = i;
}

// a particle is redrawn when a lower-numbered spine is closer than the separation
__global__ void k_conflicts(Gen g) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  const double xi = g.x[i], yi = g.y[i], pi_ = g.phi[i];
  const double Ri = radius(g, i), Ai = g.a_over_r * Ri;
  const double ux = Ai * cos(pi_), uy = Ai * sin(pi_);
  const int c = g.cell[i], cx = c % g.ng, cy = c / g.ng;
  bool bad = false;
  for (int a = -1; a <= 1 && !bad; a++)
    for (int b = -1; b <= 1 && !bad; b++) {
      const int nx = (cx + b + g.ng) % g.ng, ny = (cy + a + g.ng) % g.ng;
      const int cc = ny * g.ng + nx;
      const int s0 = g.start[cc], s1 = s0 + g.count[cc];
      for (int k = s0; k < s1; k++) {
        const int j = g.list[k];
        if (j >= i) continue;
        double dx = xi - g.x[j], dy = yi - g.y[j];
        dx -= g.L * rint(dx / g.L);
        dy -= g.L * rint(dy / g.L);
        const double Rj = radius(g, j), Aj = g.a_over_r * Rj;
        const double vx = Aj * cos(g.phi[j]), vy = Aj * sin(g.phi[j]);
        if (sc_seg::seg_seg(dx, dy, ux, uy, 0.0, 0.0, vx, vy) < g.sep * (Ri + Rj)) {
          bad = true;
          break;
        }
      }
    }
  g.redraw[i] = bad ? 1 : 0;
  if (bad) atomicAdd(g.nredraw, 1);
}

}  // namespace

extern "C" int sc_generate_packing_device(int device, int n, double packing, double a_over_r,
                                          double r_small, double r_ratio, uint64_t seed,
                                          double min_sep, double* x, double* y, double* phi,
                                          double* R, double* A, double* L_out) {
  if (n < 2 || !(packing > 0 && packing < 1) || !(a_over_r >= 0) || !(r_small > 0) ||
      !(r_ratio > 0) || !(min_sep >= 0) || !x || !y || !phi || !R || !A || !L_out)
    return SC_E_ARG;
  // shapes and box exactly as sc_generate_packing
  const double pi = 3.14159265358979323846;
  double filled = 0.0, rmax = 0.0, amax = 0.0;
  for (int i = 0; i < n; i++) {
    R[i] = (i % 2 == 0) ? r_small : r_small * r_ratio;
    A[i] = a_over_r * R[i];
    filled += pi * R[i] * R[i] + 4.0 * A[i] * R[i];
    rmax = std::fmax(rmax, R[i]);
    amax = std::fmax(amax, A[i]);
  }
  const double L = std::sqrt(filled / packing);
  *L_out = L;
  const double reach = 2.0 * amax + 2.0 * min_sep * rmax;
  int ng = (int)(L / std::fmax(reach, 1e-300));
  if (ng > 2048) ng = 2048;
  if (ng < 3) return SC_E_ARG;  // a box this small: sc_generate_packing
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return SC_E_CUDA;
  }
  Gen g{};
  g.n = n;
  g.ng = ng;
  g.L = L;
  g.gw = L / ng;
  g.sep = min_sep;
  g.a_over_r = a_over_r;
  g.r_small = r_small;
  g.r_ratio = r_ratio;
  g.seed = seed;
  const size_t N = n, NC = (size_t)ng * ng;
  void* mem = nullptr;
  const size_t bytes = 3 * N * sizeof(double) + (4 * N + 2 * NC + 1) * sizeof(int);
  cudaStream_t st = nullptr;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMallocAsync(&mem, bytes, st) != cudaSuccess) {
    if (st) cudaStreamDestroy(st);
    cudaGetLastError();
    return SC_E_NOMEM;
  }
  char* p = static_cast<char*>(mem);
  g.x = reinterpret_cast<double*>(p);
  g.y = g.x + N;
  g.phi = g.y + N;
  g.cell = reinterpret_cast<int*>(g.phi + N);
  g.rank = g.cell + N;
  g.list = g.rank + N;
  g.redraw = g.list + N;
  g.count = g.redraw + N;
  g.start = g.count + NC;
  g.nredraw = g.start + NC;
  const int B = 256, nb = (int)((N + B - 1) / B);
  std::vector<int> ones(N, 1);
  int rc = SC_OK;
  int* h_red = nullptr;
  bool ok = cudaMallocHost(&h_red, sizeof(int)) == cudaSuccess &&
            cudaMemcpyAsync(g.redraw, ones.data(), N * sizeof(int), cudaMemcpyHostToDevice,
                            st) == cudaSuccess;
  const int max_rounds = 10000;  // a packing past the placement's saturation: SC_E_NOCONV
  int round = 0;
  for (; ok && round < max_rounds; round++) {
    k_draw<<<nb, B, 0, st>>>(g, round);
    ok = cudaMemsetAsync(g.count, 0, NC * sizeof(int), st) == cudaSuccess;
    if (!ok) break;
    k_bin<<<nb, B, 0, st>>>(g);
    k_scan<<<1, 1024, 0, st>>>(g);
    k_fill<<<nb, B, 0, st>>>(g);
    ok = cudaMemsetAsync(g.nredraw, 0, sizeof(int), st) == cudaSuccess;
    if (!ok) break;
    k_conflicts<<<nb, B, 0, st>>>(g);
    ok = cudaMemcpyAsync(h_red, g.nredraw, sizeof(int), cudaMemcpyDeviceToHost, st) ==
             cudaSuccess &&
         cudaStreamSynchronize(st) == cudaSuccess;
    if (ok && *h_red == 0) break;
  }
  if (!ok)
    rc = SC_E_CUDA;
  else if (round >= max_rounds)
    rc = SC_E_NOCONV;
  if (rc == SC_OK &&
      (cudaMemcpyAsync(x, g.x, N * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
       cudaMemcpyAsync(y, g.y, N * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
       cudaMemcpyAsync(phi, g.phi, N * sizeof(double), cudaMemcpyDeviceToHost, st) !=
           cudaSuccess ||
       cudaStreamSynchronize(st) != cudaSuccess))
    rc = SC_E_CUDA;
  cudaFreeAsync(mem, st);
  cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
  if (h_red) cudaFreeHost(h_red);
  cudaGetLastError();
  return rc;
}
