// sc_pass_mixed.cu -- the mixed-precision form.
//
// State: each particle's centre is kept relative to the centre of the cell it was
// last sorted into, as an FP32 value plus an FP32 compensation term (Kahan), and
// its angle likewise; the absolute FP64 position is (col+1/2)W + x_local + x_comp,
// materialised only for the cell sort, the Lees-Edwards set-back and for output.
// Pair geometry and forces are FP32, and no FP64 instruction runs in the force
// passes.  On the steps that record stress and energy, those come from an FP64
// evaluation of the state (k_mx_se64, sc_pass64.cu), so they differ from the FP64
// form's only through the state itself.
//
// Neighbour list: every pair whose spines, in the Lees-Edwards frame of the build,
// are closer than R_i + R_j + pad (the capsule distance; FP32, bound inflated by
// 2e-5 relative plus 1e-5).  It is rebuilt when a particle's spine has moved since
// the build (centre displacement plus A times the rotation), plus this step's move
// as an allowance for the next predictor excursion, by half of what is left of the
// padding once the shear accumulated since the build, |gamma - gamma_build|
// (S_max + pad), is taken off.  Then no pair outside the list can come into
// contact, so the set of interacting pairs is exactly the reference's (whose own
// padded list is larger).
// Each entry packs the neighbour's slot with the cell offset (dc, dr) between the
// two cells, so the displacement is rec_i - rec_j - (dc W, dr H) with no box
// length in the FP32 arithmetic.
//
// Force pass: one thread per list position gathers over its particle's list and
// evaluates each pair from its own side.
#include "sc_fire.cuh"
#include "sc_internal.hpp"
#include "sc_pair.cuh"

namespace sc {

namespace {

__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
  float y = v + c;
  float t = s + y;
  c = y - (t - s);
  s = t;
}

// Affine step of a compensated coordinate, with g the increment of the scale
// (the factor is 1 + g): (s + c) <- (s + c + v)(1 + g) when the increment v is
// scaled too (resize), (s + c)(1 + g) + v when it is not (pure shear).  The
// affine part (s + c + v) g is small, so it is added to the increment before the
// compensated sum and the FP32 factor's rounding never touches s itself.
template <bool SCALE_V>
__device__ __forceinline__ void kahan_affine(float& s, float& c, float v, float g) {
  float y = v + c;
  y = fmaf(SCALE_V ? s + y : s + c, g, y);
  float t = s + y;
  c = y - (t - s);
  s = t;
}

// The Heun step of one particle after its forces (fx, fy, tq) at the pass's
// positions are known: the predictor (MODE 2, 4) or corrector (MODE 1, 3) with the
// compensated FP32 state, the rebuild test, or (MODE 0) the forces alone.  ri is
// the particle's record at the pass's positions, gam the pass's gamma.
template <int MODE>
__device__ __forceinline__ void mixed_epilogue(const Dev& d, const StepScalars& ts,
                                               const SysGeom& g, int s, int i, float4 ri,
                                               float4 pai, float gam, float fx, float fy,
                                               float tq) {
  const float dt = ts.f_step;
  const float A = pai.y, invI = pai.w;
  if (MODE == PASS_FORCE) {
    d.fx[i] = fx;
    d.fy[i] = fy;
    d.tau[i] = tq;
  } else if (MODE == PASS_PRED_STRAIN || MODE == PASS_PRED_RESIZE) {
    const float4 c = d.mc[i];
    float v0x, v0y, v0p;
    if (MODE == PASS_PRED_STRAIN) {
      // strain_step predictor, strain_dynamics.cpp:187-199
      float phi = c.z + c.w;
      const float RC = d.rcf[i];
      v0x = fx - gam * fy;
      v0y = fy;
      v0p = tq * invI - ts.f_rate * (0.5f * (1.f - RC * __cosf(2.f * phi)));
    } else {
      // resize_step predictor, resize_dynamics.cpp:172-191
      v0x = fx;
      v0y = fy;
      v0p = tq * invI;
    }
    // pure shear: isolated rotation in the flow (+x/2, -y/2) at the strain rate
    // (pure_euler_est_2p, src/cuda/2point_dynamics.cu:1889-1891)
    const float rot = (MODE == PASS_PRED_RESIZE && ts.mode == 3)
                          ? ts.f_rate * (-0.5f * d.rcf[i] * __sinf(2.f * (c.z + c.w)))
                          : 0.f;
    float xt = ri.x + (c.x + dt * v0x);
    float yt = ri.y + (c.y + dt * v0y);
    float pt = c.z + (c.w + dt * (v0p + rot));
    if (MODE == PASS_PRED_RESIZE) {
      // about the cell centre, which moves with the same affine map
      if (ts.mode == 3) {
        xt = fmaf(ri.x + c.x, ts.f_gx, xt);  // the flow acts on the pre-step position
        yt = fmaf(ri.y + c.y, ts.f_gy, yt);
      } else {
        xt = fmaf(xt, ts.f_gx, xt);  // resize scales the moved position
        yt = fmaf(yt, ts.f_gy, yt);
      }
    }
    float sn, cs;
    sincosf(pt, &sn, &cs);
    d.rec_t[i] = make_float4(xt, yt, A * cs, A * sn);
    // pure shear keeps the rotation rate of the flow in place of the predicted angle
    d.mv[i] = make_float4(v0x, v0y, v0p, (MODE == PASS_PRED_RESIZE && ts.mode == 3) ? rot : pt);
  } else {
    const float4 v0 = d.mv[i];
    float4 c = d.mc[i];
    float4 r = d.rec[i];
    float ddx, ddy, ddp;
    if (MODE == PASS_CORR_STRAIN) {
      // strain_step corrector, strain_dynamics.cpp:203-219
      const float RC = d.rcf[i];
      float v1x = fx - gam * fy;
      float v1y = fy;
      float v1p = tq * invI - ts.f_rate * (0.5f * (1.f - RC * __cosf(2.f * v0.w)));
      ddx = 0.5f * dt * (v0.x + v1x);
      ddy = 0.5f * dt * (v0.y + v1y);
      ddp = 0.5f * dt * (v0.z + v1p);
    } else {
      // resize_step corrector, resize_dynamics.cpp:194-218.  Pure shear
      // (pure_heun_corr_2p, src/cuda/2point_dynamics.cu:2140-2173) ends at the
      // predicted state plus dt/2 (F~ - F0): the same Heun mean of the contact
      // forces, with the flow's displacement and rotation taken by Euler.
      ddx = 0.5f * dt * (v0.x + fx);
      ddy = 0.5f * dt * (v0.y + fy);
      ddp = 0.5f * dt * (v0.z + tq * invI);
      if (ts.mode == 3) ddp = fmaf(dt, v0.w, ddp);
    }
    float4 m = d.mm[i];
    float aff = 0.f;  // the next step's affine displacement, for the rebuild test
    if (MODE == PASS_CORR_RESIZE) {
      const float gx = ts.f_gx, gy = ts.f_gy;
      const int cp = d.cellp[i];
      // the cell centre moves with the affine map as well
      float cx = ((float)(cp & 0xffff) + 0.5f) * ts.f_Wc;
      float cy = ((float)(cp >> 16) + 0.5f) * ts.f_Hc;
      float x0 = r.x, y0 = r.y;
      if (ts.mode == 3) {
        kahan_affine<false>(r.x, c.x, ddx, gx);
        kahan_affine<false>(r.y, c.y, ddy, gy);
      } else {
        kahan_affine<true>(r.x, c.x, ddx, gx);
        kahan_affine<true>(r.y, c.y, ddy, gy);
      }
      m.x += (r.x - x0) + cx * gx;
      m.y += (r.y - y0) + cy * gy;
      aff = fabsf((cx + r.x) * gx) + fabsf((cy + r.y) * gy);
    } else {
      kahan_add(r.x, c.x, ddx);
      kahan_add(r.y, c.y, ddy);
      m.x += ddx;
      m.y += ddy;
    }
    kahan_add(c.z, c.w, ddp);
    float sn, cs;
    sincosf(c.z + c.w, &sn, &cs);
    r.z = A * cs;
    r.w = A * sn;
    d.rec[i] = r;
    d.mc[i] = c;
    d.mm[i] = m;
    if (!(isfinite(r.x) && isfinite(r.y) && isfinite(c.z))) atomicOr(d.status, ST_NAN);
    // padding left after the shear since the list was built (next corrector's gamma)
    float dg = fabsf(ts.f_gamma_p - d.gbuild[s]) + 2.f * fabsf(ts.f_rate * dt);
    float h = 0.5f * (g.fpad - dg * (g.smax + g.fpad));
    // a spine end moves by at most the centre's displacement plus A times the
    // rotation; the next step's move is allowed for as well
    float reach = sqrtf(m.x * m.x + m.y * m.y) + A * fabsf((c.z + c.w) - m.z) +
                  sqrtf(ddx * ddx + ddy * ddy) + aff + A * fabsf(ddp);
    if (!(reach < h)) request_rebuild(d, s);
  }
}

// The force pass of one list position (the per-particle pass): the particle's
// pairs from its own side over its full list, then the Heun epilogue.  COH: the
// records were written by other blocks of the same (persistent) launch, so they are
// loaded through L2 (ld.global.cg) and never through the read-only path, which holds
// only data that stays unchanged for a whole launch.
template <int MODE, bool TWO, bool COH = false>
__device__ __forceinline__ void pass_mixed_position(const Dev& d,
                                                    const StepScalars* __restrict__ tab,
                                                    int row, int pos) {
  constexpr bool kPred = (MODE == PASS_CORR_STRAIN || MODE == PASS_CORR_RESIZE);
  const int i = d.ord[pos];  // the slot this thread works on (lists ordered by length)
  const int s = d.psys[i];
  if (d.skip && d.skip[s]) return;  // a converged minimiser system
  const SysGeom& g = d.geom[s];
  const StepScalars& ts = tab[row * d.nsys + s];
  const float4* __restrict__ REC = kPred ? d.rec_t : d.rec;
  const float W = kPred ? ts.f_Wc : ts.f_Wp;
  const float H = kPred ? ts.f_Hc : ts.f_Hp;
  const float gam = kPred ? ts.f_gamma_c : ts.f_gamma_p;
  const bool smallx = g.cols < 3, smally = g.rows < 3;
  const float Lxf = W * g.cols, Lyf = H * g.rows;
  constexpr bool two_point = TWO;

#define SC_REC(k) (COH ? __ldcg(REC + (k)) : REC[(k)])
  const float4 ri = SC_REC(i);
  const float4 pai = d.pa[i];  // (R, A, index bits, 1/I)
  const int cnt = d.nbr_pn[pos];
  // the list is column-major: entry k of this slot sits k * ntot words further on;
  // Lst walks it, two entries ahead of the pair being computed
  const unsigned* __restrict__ Lst = reinterpret_cast<const unsigned*>(d.nbr_p) + pos;
  const int stride = d.ntot;

  float fx = 0.f, fy = 0.f, tq = 0.f;
  // software pipeline: the list entry two ahead and the neighbour data one ahead
  // are in flight while the current pair is computed
  unsigned e1 = cnt > 0 ? __ldg(Lst) : 0u;
  Lst += stride;
  unsigned e2 = cnt > 1 ? __ldg(Lst) : 0u;
  // the neighbour's record and radius (its A^2 is |shaft|^2 from the record)
  float4 r1 = make_float4(0.f, 0.f, 0.f, 0.f);
  float R1 = 0.f;
  if (cnt > 0) {
    r1 = SC_REC(e1 & kSlotMask);
    R1 = d.rf[e1 & kSlotMask];
  }
  const float ai = pai.y * pai.y;
  for (int k = 0; k < cnt; k++) {
    const unsigned e = e1;
    const float4 rj = r1;
    const float Rj = R1;
    e1 = e2;
    if (k + 1 < cnt) {
      r1 = SC_REC(e1 & kSlotMask);
      R1 = d.rf[e1 & kSlotMask];
    }
    Lst += stride;
    if (k + 2 < cnt) e2 = __ldg(Lst);
    float dx = ri.x - rj.x + (float)(1 - (int)((e >> 28) & 3u)) * W;
    float dy = ri.y - rj.y + (float)(1 - (int)(e >> 30)) * H;
    if (smallx) dx += Lxf * (float)((dx < -0.5f * Lxf) - (dx > 0.5f * Lxf));
    if (smally) dy += Lyf * (float)((dy < -0.5f * Lyf) - (dy > 0.5f * Lyf));
    // Each thread evaluates the pair from its own particle's side (i as "p"): the
    // forces need no canonical order, the two evaluations of a pair differ only by
    // FP32 rounding.  Stress and energy are not summed here: on the steps that
    // record them they come from the FP64 evaluation of the state (k_mx_se64).
    PairF32 o;
    const float cj = fmaf(rj.z, rj.z, rj.w * rj.w);
    const bool touch =
        two_point ? pair2_fp32(dx, dy, ri.z, ri.w, ai, rj.z, rj.w, cj, pai.x + Rj, gam, o)
                  : pair_fp32<false>(dx, dy, ri.z, ri.w, ai, rj.z, rj.w, cj, pai.x + Rj, gam,
                                     false, o);
    if (!touch) continue;
    fx += o.fx;
    fy += o.fy;
    tq += o.tp;
  }

#undef SC_REC
  mixed_epilogue<MODE>(d, ts, g, s, i, ri, pai, gam, fx, fy, tq);
}

template <int MODE, bool TWO>
__global__ void __launch_bounds__(128, TWO ? 6 : 12) k_pass_mixed(Dev d,
                                                       const StepScalars* __restrict__ tab,
                                                       int row) {
  constexpr bool kPred = (MODE == PASS_CORR_STRAIN || MODE == PASS_CORR_RESIZE);
  if (kPred) mark_pending_rebuilds(d, tab, row);
  const int pos = blockIdx.x * blockDim.x + threadIdx.x;
  if (pos >= d.ntot) return;
  pass_mixed_position<MODE, TWO>(d, tab, row, pos);
}

// ---- persistent shear steps ----
//
// For small and medium systems a step's two passes are short next to their launch
// and the gaps between launches.  One cooperative launch (every block resident, so a
// grid barrier cannot wait for a block that never runs) advances several steps:
// the corrector pass over all positions, a grid barrier, the predictor pass, a grid
// barrier.  A step whose corrector requests a rebuild (or whose row sets gamma back)
// ends the launch after that corrector; the host runs the rebuild and the predictor
// and relaunches.  Every wait is bounded (kBarrierSpins): a barrier that times out
// records ST_BARRIER_TIMEOUT, which the host reports as an error.

// generation barrier over all blocks of the grid (thread 0 of each block arrives)
__device__ __forceinline__ void grid_barrier(unsigned* bar, int* status) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* vgen = bar + 1;
    const unsigned gen = *vgen;
    __threadfence();
    if (atomicAdd(bar, 1u) == gridDim.x - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      unsigned it = 0;
      while (*vgen == gen) {
        if (++it > kBarrierSpins) {
          atomicOr(status, ST_BARRIER_TIMEOUT);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
}

template <bool TWO>
__global__ void __launch_bounds__(128, TWO ? 6 : 12) k_persist_steps(
    Dev d, const StepScalars* __restrict__ tab, int row0, int nsteps, int* out) {
  const int stride = gridDim.x * blockDim.x;
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
  int k = 0, stopped = 0;
  for (; k < nsteps; k++) {
    const int row = row0 + k;
    // systems that set gamma back at this step rebuild after its corrector
    if (blockIdx.x == 0)
      for (int s = threadIdx.x; s < d.nsys; s += blockDim.x)
        if (tab[row * d.nsys + s].setback) {
          atomicOr(&d.flags[s], 2);
          atomicExch(d.any, 1);
        }
    for (int pos = t0; pos < d.ntot; pos += stride)
      pass_mixed_position<PASS_CORR_STRAIN, TWO, true>(d, tab, row, pos);
    grid_barrier(d.gbar, d.status);
    if (*(volatile int*)d.any != 0) {  // the same value in every block after the barrier
      stopped = 1;
      break;
    }
    for (int pos = t0; pos < d.ntot; pos += stride)
      pass_mixed_position<PASS_PRED_STRAIN, TWO, true>(d, tab, row, pos);
    grid_barrier(d.gbar, d.status);
  }
  if (t0 == 0) *out = 2 * k + stopped;
}

// ---- persistent FIRE ----
//
// FIRE iterations of the mixed form in one cooperative launch: the force pass over
// all positions, the chunk partials, the per-system FIRE update and the particle
// update, each followed by a grid barrier.  The blocks have the 256 threads of the
// launch-per-kernel reductions (k_fire_chunk), so each chunk sums in the same order
// and the iterates equal those of the graph and eager paths bit for bit.  The launch
// ends after `iters` iterations, after the iteration whose update asks for a
// rebuild (the host runs it), or at the iteration in which the last system
// converges: *out = 4 * iterations + (0 all ran, 1 rebuild pending, 2 all converged).
static_assert(fire::kFireBlock == 256, "the persistent FIRE blocks are the reduction blocks");

template <bool TWO>
__global__ void __launch_bounds__(256, TWO ? 3 : 4) k_persist_fire(
    Dev d, FireState f, const StepScalars* __restrict__ tab, double ftol, double dt_max,
    int iters, int* out) {
  const int stride = gridDim.x * blockDim.x;
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
  int k = 0, why = 0;
  while (k < iters) {
    for (int pos = t0; pos < d.ntot; pos += stride)
      pass_mixed_position<PASS_FORCE, TWO, true>(d, tab, 0, pos);
    grid_barrier(d.gbar, d.status);
    for (int ch = blockIdx.x; ch < d.npchunks; ch += gridDim.x) {
      fire::fire_chunk<true>(d, f, ch);
      __syncthreads();  // the next chunk reuses the block's shared partials
    }
    grid_barrier(d.gbar, d.status);
    // one block per system, as k_fire_sys (the block has kFireBlock threads)
    for (int s = blockIdx.x; s < d.nsys; s += gridDim.x) fire::fire_sys(d, f, s, ftol, dt_max);
    grid_barrier(d.gbar, d.status);
    k++;
    // every block sees the same flags: they change only in the phase before the barrier
    int pending = 0;
    for (int s = threadIdx.x; s < d.nsys; s += blockDim.x) pending |= (__ldcg(f.done + s) == 0);
    if (!__syncthreads_or(pending)) {
      why = 2;
      break;
    }
    for (int i = t0; i < d.ntot; i += stride) fire::fire_update<true>(d, f, i);
    grid_barrier(d.gbar, d.status);
    if (*(volatile int*)d.any != 0) {
      why = 1;
      break;
    }
  }
  if (t0 == 0) *out = 4 * k + why;
}

template <int MODE>
void launch_one(const Dev& d, const StepScalars* tab, int row, cudaStream_t st, int block) {
  int grid = (d.ntot + block - 1) / block;
  if (d.contact_model == 1)
    k_pass_mixed<MODE, true><<<grid, block, 0, st>>>(d, tab, row);
  else
    k_pass_mixed<MODE, false><<<grid, block, 0, st>>>(d, tab, row);
}

// ---- tile force pass ----
//
// One block per tile of cells (a contiguous range of slots).  The tile's records
// and radii are staged in shared memory.  Its compute entries, ordered by owner,
// hold every pair of an owner with a partner outside the tile and every pair with
// a partner of higher slot inside it, so a pair inside the tile is evaluated once:
// the threads take the entries in turn (one pair per thread, whatever the list
// lengths) and leave each pair's forces and both torques in shared memory; then
// each owner sums its own entries in list order and, with the opposite sign, the
// entries of the pairs whose lower partner computed them (its read entries, in
// list order).  The sums are deterministic.  A tile with more particles or pair
// entries than shared memory holds uses global memory for the excess.
template <int MODE, bool TWO>
__global__ void __launch_bounds__(kTileThreads, TWO ? 2 : 4) k_tile_pass(
    Dev d, const StepScalars* __restrict__ tab, int row) {
  constexpr bool kCorr = (MODE == PASS_CORR_STRAIN || MODE == PASS_CORR_RESIZE);
  if (kCorr) mark_pending_rebuilds(d, tab, row);
  __shared__ float4 s_rec[kTileCap];
  __shared__ float s_R[kTileCap];
  __shared__ float4 s_pb[kTilePairCap];
  const int4 ti = d.tinfo[blockIdx.x];
  const int p0 = ti.x, nown = ti.y, ne = ti.z;
  if (nown <= 0) return;
  const int s = d.psys[p0];
  if (d.skip && d.skip[s]) return;  // a converged minimiser system (the whole block)
  const SysGeom& g = d.geom[s];
  const StepScalars& ts = tab[row * d.nsys + s];
  const float4* __restrict__ REC = kCorr ? d.rec_t : d.rec;
  const float W = kCorr ? ts.f_Wc : ts.f_Wp;
  const float H = kCorr ? ts.f_Hc : ts.f_Hp;
  const float gam = kCorr ? ts.f_gamma_c : ts.f_gamma_p;
  const bool smallx = g.cols < 3, smally = g.rows < 3;
  const float Lxf = W * g.cols, Lyf = H * g.rows;
  const int nst = nown < kTileCap ? nown : kTileCap;
  for (int l = threadIdx.x; l < nst; l += blockDim.x) {
    s_rec[l] = REC[p0 + l];
    s_R[l] = d.rf[p0 + l];
  }
  float4* pb = ne <= kTilePairCap ? s_pb : d.t_pb + (size_t)p0 * kTileEPP;
  const size_t ebase = (size_t)p0 * kTileEPP;
  __syncthreads();
  for (int e = threadIdx.x; e < ne; e += blockDim.x) {
    const int o = d.t_own[ebase + e];
    const unsigned pe = d.t_pe[ebase + e];
    const float4 ri = o < kTileCap ? s_rec[o] : REC[p0 + o];
    const float Ri = o < kTileCap ? s_R[o] : d.rf[p0 + o];
    const unsigned pl = pe & kTilePayload;
    float4 rj;
    float Rj;
    if (pe & kTileInt) {
      rj = pl < (unsigned)kTileCap ? s_rec[pl] : REC[p0 + pl];
      Rj = pl < (unsigned)kTileCap ? s_R[pl] : d.rf[p0 + pl];
    } else {
      rj = REC[pl];
      Rj = d.rf[pl];
    }
    float dx = ri.x - rj.x + (float)(1 - (int)((pe >> 28) & 3u)) * W;
    float dy = ri.y - rj.y + (float)(1 - (int)(pe >> 30)) * H;
    if (smallx) dx += Lxf * (float)((dx < -0.5f * Lxf) - (dx > 0.5f * Lxf));
    if (smally) dy += Lyf * (float)((dy < -0.5f * Lyf) - (dy > 0.5f * Lyf));
    PairF32 res;
    const float ai = fmaf(ri.z, ri.z, ri.w * ri.w);
    const float cj = fmaf(rj.z, rj.z, rj.w * rj.w);
    const bool touch =
        TWO ? pair2_fp32(dx, dy, ri.z, ri.w, ai, rj.z, rj.w, cj, Ri + Rj, gam, res)
            : pair_fp32<false>(dx, dy, ri.z, ri.w, ai, rj.z, rj.w, cj, Ri + Rj, gam, false,
                               res);
    pb[e] = touch ? make_float4(res.fx, res.fy, res.tp, res.tq) : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  __syncthreads();
  for (int l = threadIdx.x; l < nown; l += blockDim.x) {
    const int i = p0 + l;
    const int2 m = d.t_meta[i];
    const int c0 = m.x & 0xffffff, nc = (int)((unsigned)m.x >> 24);
    const int r0 = m.y & 0xffffff, nr = (int)((unsigned)m.y >> 24);
    float fx = 0.f, fy = 0.f, tq = 0.f;
    // (the bounds only bite after a list overflow, which the status reports)
    for (int k = 0; k < nc && c0 + k < ne; k++) {
      const float4 v = pb[c0 + k];
      fx += v.x;
      fy += v.y;
      tq += v.z;
    }
    for (int k = 0; k < nr && r0 + k < ti.w; k++) {
      const unsigned e = d.t_rd[ebase + r0 + k];
      if (e >= (unsigned)ne) continue;  // kTileNoEntry: a pair nobody computes
      const float4 v = pb[e];
      fx -= v.x;
      fy -= v.y;
      tq += v.w;
    }
    const float4 ri = l < kTileCap ? s_rec[l] : REC[i];
    mixed_epilogue<MODE>(d, ts, g, s, i, ri, d.pa[i], gam, fx, fy, tq);
  }
}

template <int MODE>
void launch_tile(const Dev& d, const StepScalars* tab, int row, cudaStream_t st) {
  if (d.contact_model == 1)
    k_tile_pass<MODE, true><<<d.ntiles, kTileThreads, 0, st>>>(d, tab, row);
  else
    k_tile_pass<MODE, false><<<d.ntiles, kTileThreads, 0, st>>>(d, tab, row);
}

// block-wide exclusive scan of one int per thread; *total the block's sum
__device__ __forceinline__ int tile_excl_scan(int v, int* sh, int* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[w] = x;
  __syncthreads();
  if (w == 0) {
    int t = lane < nw ? sh[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    sh[lane] = t;
  }
  __syncthreads();
  const int excl = x - v + (w > 0 ? sh[w - 1] : 0);
  *total = sh[nw - 1];
  __syncthreads();
  return excl;
}

// The tile lists of the rebuilt systems from their mixed lists (one block per
// tile): each particle's entries split into compute entries (partner outside the
// tile, or inside it at a higher slot) and read entries (inside, at a lower slot);
// offsets by block scans; then every read entry finds the compute entry of its pair
// among the partner's.  A pair listed by one side only (the capsule test's rounding
// at the padding's edge, far from contact) is computed by nobody.
__global__ void __launch_bounds__(kTileThreads) k_tile_lists(Dev d, int all) {
  if (!all && *d.any == 0) return;
  const int4 tl = d.tiles[blockIdx.x];
  if (!all && d.flags[tl.x] == 0) return;
  __shared__ int sh[32];
  const int cl = tl.y + tl.z - 1;
  const int p0 = d.cell_start[tl.y];
  const int p1 = d.cell_start[cl] + d.cell_count[cl];
  const int nown = p1 - p0;
  const size_t ebase = (size_t)p0 * kTileEPP;
  const int ecap = nown * kTileEPP;
  const int ntot = d.ntot;
  int cc = 0, cr = 0;  // running offsets (the same in every thread)
  bool over = false;
  for (int base = 0; base < nown; base += blockDim.x) {
    const int l = base + threadIdx.x;
    int nc = 0, nr = 0;
    if (l < nown) {
      const int i = p0 + l;
      const int cnt = min(d.nbr_n[i], d.maxn);
      for (int k = 0; k < cnt; k++) {
        const int j = (int)((unsigned)d.nbr[(size_t)k * ntot + i] & kSlotMask);
        if (j >= p0 && j < p1 && j - p0 < l)
          nr++;
        else
          nc++;
      }
      over = over || nc > 255 || nr > 255 || nown > 65535;
    }
    int tc, tr;
    const int ec = tile_excl_scan(nc, sh, &tc);
    const int er = tile_excl_scan(nr, sh, &tr);
    if (l < nown) d.t_meta[p0 + l] = make_int2((cc + ec) | (nc << 24), (cr + er) | (nr << 24));
    cc += tc;
    cr += tr;
  }
  over = __syncthreads_or(over) != 0;
  if (cc > ecap || cr > ecap || over) {
    if (threadIdx.x == 0) atomicOr(d.status, ST_NBR_OVERFLOW);
    cc = min(cc, ecap);
    cr = min(cr, ecap);
  }
  if (threadIdx.x == 0) d.tinfo[blockIdx.x] = make_int4(p0, nown, cc, cr);
  for (int l = threadIdx.x; l < nown; l += blockDim.x) {
    const int i = p0 + l;
    const int cnt = min(d.nbr_n[i], d.maxn);
    int q = d.t_meta[i].x & 0xffffff;
    for (int k = 0; k < cnt; k++) {
      const unsigned e = (unsigned)d.nbr[(size_t)k * ntot + i];
      const int j = (int)(e & kSlotMask);
      const bool in = j >= p0 && j < p1;
      if (in && j - p0 < l) continue;
      if (q < ecap) {
        d.t_own[ebase + q] = (unsigned short)l;
        d.t_pe[ebase + q] = (e & ~kSlotMask) | (in ? (kTileInt | (unsigned)(j - p0)) : (unsigned)j);
      }
      q++;
    }
  }
  __syncthreads();  // every compute entry of the tile is written
  for (int l = threadIdx.x; l < nown; l += blockDim.x) {
    const int i = p0 + l;
    const int cnt = min(d.nbr_n[i], d.maxn);
    int r = d.t_meta[i].y & 0xffffff;
    for (int k = 0; k < cnt; k++) {
      const int j = (int)((unsigned)d.nbr[(size_t)k * ntot + i] & kSlotMask);
      if (!(j >= p0 && j < p1 && j - p0 < l)) continue;
      const int2 m = d.t_meta[j];
      const int q0 = m.x & 0xffffff, qn = (int)((unsigned)m.x >> 24);
      unsigned found = kTileNoEntry;
      for (int q = q0; q < q0 + qn && q < ecap; q++)
        if ((d.t_pe[ebase + q] & (kTileInt | kTilePayload)) == (kTileInt | (unsigned)l)) {
          found = (unsigned)q;
          break;
        }
      if (r < ecap) d.t_rd[ebase + r] = found;
      r++;
    }
  }
}

// ---- rebuild support ----

// FP64 absolute state from the compensated local state (flagged systems, systems
// that set back gamma at this step, or all).
// FP64 state of slot i from its compensated record and its cell centre
__device__ __forceinline__ void materialize_slot(const Dev& d, const StepScalars& ts, int i) {
  int cp = d.cellp[i];
  float4 r = d.rec[i];
  float4 c = d.mc[i];
  double x = ((cp & 0xffff) + 0.5) * ts.W_p + ((double)r.x + (double)c.x);
  double y = ((cp >> 16) + 0.5) * ts.H_p + ((double)r.y + (double)c.y);
  d.xy[i] = make_double2(x, y);
  d.ph[i] = (double)c.z + (double)c.w;
}

// every slot (all) or, after launch_rb_worklist, the slots of the listed systems
__global__ void k_mx_materialize(Dev d, const StepScalars* __restrict__ tab, int row, int all) {
  if (all) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < d.ntot) materialize_slot(d, tab[row * d.nsys + d.psys[i]], i);
    return;
  }
  for_listed_slots(d, [&](int i, int s) { materialize_slot(d, tab[row * d.nsys + s], i); });
}

// Compensated local state from the FP64 state after a cell sort.
__global__ void k_mx_local(Dev d, const StepScalars* __restrict__ tab, int row, int all) {
  if (!all && *d.any == 0) return;
  for_slots(d, all != 0, [&](int i, int s) {
    const SysGeom& g = d.geom[s];
    const StepScalars& ts = tab[row * d.nsys + s];
    int lc = d.cell[i] - g.c0;
    int col, rw;
    cell_colrow(g, lc, &col, &rw);
    d.cellp[i] = col | (rw << 16);
    double2 p = d.xy[i];
    double lx = p.x - (col + 0.5) * ts.W_p;
    double ly = p.y - (rw + 0.5) * ts.H_p;
    double phi = d.ph[i];
    float xl = (float)lx, yl = (float)ly, pf = (float)phi;
    double2 ra = d.ra[i];
    double2 irc = d.irc[i];
    float A = (float)ra.y;
    float sn, cs;
    sincosf(pf, &sn, &cs);
    d.rec[i] = make_float4(xl, yl, A * cs, A * sn);
    d.mc[i] = make_float4((float)(lx - xl), (float)(ly - yl), pf, (float)(phi - pf));
    d.mm[i] = make_float4(0.f, 0.f, pf + (float)(phi - pf), 0.f);
    // 1/I in FP32 (an FP64 division per particle costs more than the whole record)
    d.pa[i] = make_float4((float)ra.x, A, __int_as_float(d.id[i]), __frcp_rn((float)irc.x));
    d.rcf[i] = (float)irc.y;
    d.rf[i] = (float)ra.x;
  });
}

// The padded neighbour list in FP32 (see the file comment).  Two stages per
// particle: the centre-distance test over the candidates of the 3x3 cells, whose
// survivors (about a third) are queued in scan order, and the capsule test over the
// queue.  Threads of a warp then run the expensive test about as often as their own
// survivors need, not once per candidate of the slowest lane; the list order (cell
// by cell, slots ascending) is the scan order either way.
constexpr int kMxQueue = 24;

// The list of slot i (system s): see the file comment and kMxQueue.
__device__ __forceinline__ void build_list_slot(const Dev& d, const StepScalars* __restrict__ tab,
                                                int row, int i, int s) {
  const SysGeom& g = d.geom[s];
  const StepScalars& ts = tab[row * d.nsys + s];
  const float W = ts.f_Wp, H = ts.f_Hp, gam = ts.f_gamma_p, pad = (float)g.pad;
  const float Lxf = W * g.cols, Lyf = H * g.rows;
  const int cp = d.cellp[i];
  const int col = cp & 0xffff, rw = cp >> 16;
  const float4 ri = d.rec[i];
  const float2 rai = reinterpret_cast<const float2*>(d.pa)[2 * (size_t)i];  // (R, A)
  const int ncx = g.cols < 3 ? g.cols : 3, ncy = g.rows < 3 ? g.rows : 3;
  const bool smallx = ncx < 3, smally = ncy < 3;
  unsigned queue[kMxQueue];  // survivors of the centre test: slot | cell offset code
  int nq = 0, cnt = 0;
  // capsule test of the queued candidates, accepted ones appended in queue order
  auto flush = [&]() {
    for (int q = 0; q < nq; q++) {
      const unsigned e = queue[q];
      const int j = (int)(e & kSlotMask);
      const float4 rj = d.rec[j];
      const float Rj = d.rf[j];
      float dx = ri.x - rj.x + (float)(1 - (int)((e >> 28) & 3u)) * W;
      float dy = ri.y - rj.y + (float)(1 - (int)(e >> 30)) * H;
      if (smallx) dx += Lxf * (float)((dx < -0.5f * Lxf) - (dx > 0.5f * Lxf));
      if (smally) dy += Lyf * (float)((dy < -0.5f * Lyf) - (dy > 0.5f * Lyf));
      if (capsules_within(fmaf(gam, dy, dx), dy, ri.z, ri.w, rj.z, rj.w,
                          (rai.x + Rj + pad) * 1.00002f + 1e-5f)) {
        if (cnt < d.maxn) d.nbr[(size_t)cnt * d.ntot + i] = (int)e;
        cnt++;
      }
    }
    nq = 0;
  };
  for (int a = 0; a < ncy; a++) {
    int dr = smally ? a - rw : a - 1;
    int r2 = smally ? a : wrap_index(rw + dr, g.rows);
    for (int b = 0; b < ncx; b++) {
      int dc = smallx ? b - col : b - 1;
      int c2 = smallx ? b : wrap_index(col + dc, g.cols);
      int cc = g.c0 + cell_local(g, c2, r2);
      int st = d.cell_start[cc], en = st + d.cell_count[cc];
      unsigned code = ((unsigned)(dc + 1) << 28) | ((unsigned)(dr + 1) << 30);
      const float ox = (float)dc * W, oy = (float)dr * H;
      for (int j = st; j < en; j++) {
        if (j == i) continue;
        const float4 rj = d.rec[j];
        const float2 raj = reinterpret_cast<const float2*>(d.pa)[2 * (size_t)j];
        float dx = ri.x - rj.x - ox;
        float dy = ri.y - rj.y - oy;
        if (smallx) dx += Lxf * (float)((dx < -0.5f * Lxf) - (dx > 0.5f * Lxf));
        if (smally) dy += Lyf * (float)((dy < -0.5f * Lyf) - (dy > 0.5f * Lyf));
        const float lim = (rai.x + rai.y + raj.x + raj.y + pad) * 1.00002f + 1e-6f;
        const float dxl = fmaf(gam, dy, dx);
        if (dxl * dxl + dy * dy < lim * lim) {
          queue[nq++] = (unsigned)j | code;
          if (nq == kMxQueue) flush();
        }
      }
    }
  }
  flush();
  d.nbr_n[i] = cnt;
  if (cnt > d.maxn) atomicOr(d.status, ST_NBR_OVERFLOW);
  if (i == g.p0) d.gbuild[s] = gam;
}

__global__ void __launch_bounds__(128, 12) k_mx_build_list(Dev d, const StepScalars* __restrict__ tab,
                                                      int row, int all) {
  if (!all && *d.any == 0) return;
  for_slots(d, all != 0, [&](int i, int s) { build_list_slot(d, tab, row, i, s); });
}

// Force-pass ordering: within each window of kOrderWindow slots, a stable sort
// of the slots by list length; the lists are copied to their positions.  A window
// is redone when any of its slots belongs to a system that was rebuilt.
__device__ __forceinline__ void order_window(const Dev& d, int base, int i, bool valid) {
  __shared__ int len[kOrderWindow];
  int c = 0x7fffffff;  // slots past the end sort last
  if (valid) c = min(d.nbr_n[i], d.maxn);
  len[threadIdx.x] = c;
  __syncthreads();
  int rank = 0;
  for (int k = 0; k < kOrderWindow; k++) {
    const int o = len[k];
    rank += (o < c) | ((o == c) & (k < (int)threadIdx.x));
  }
  if (!valid) return;
  const int pos = base + rank;
  d.ord[pos] = i;
  d.nbr_pn[pos] = c;
  const size_t n = d.ntot;
  for (int k = 0; k < c; k++) d.nbr_p[k * n + pos] = d.nbr[k * n + i];
}

__global__ void __launch_bounds__(kOrderWindow) k_mx_order(Dev d, int all) {
  if (!all && *d.any == 0) return;
  const int base = blockIdx.x * kOrderWindow;
  const int i = base + threadIdx.x;
  const bool valid = i < d.ntot;
  const bool mine = valid && (all || d.flags[d.psys[i]] != 0);
  if (!__syncthreads_or(mine)) return;
  order_window(d, base, i, valid);
}

// The list build and the force-pass ordering fused (the per-particle pass), one
// block per window of kOrderWindow slots: the window's slots of rebuilt systems
// build their lists, then the window is ordered and its lists copied to their
// positions while they are still in cache.  Same lists and order as
// k_mx_build_list followed by k_mx_order.
__global__ void __launch_bounds__(kOrderWindow, 12) k_mx_build_order(
    Dev d, const StepScalars* __restrict__ tab, int row, int all) {
  if (!all && *d.any == 0) return;
  const int base = blockIdx.x * kOrderWindow;
  const int i = base + threadIdx.x;
  const bool valid = i < d.ntot;
  const int s = valid ? d.psys[i] : 0;
  const bool mine = valid && (all || d.flags[s] != 0);
  if (!__syncthreads_or(mine)) return;
  if (mine) build_list_slot(d, tab, row, i, s);
  __syncthreads();  // the window's lengths and lists are complete
  order_window(d, base, i, valid);
}

inline int nblk(int n, int b) { return (n + b - 1) / b; }

}  // namespace

void launch_mx_order(const Dev& d, bool all, cudaStream_t st) {
  k_mx_order<<<nblk(d.ntot, kOrderWindow), kOrderWindow, 0, st>>>(d, all ? 1 : 0);
}

void launch_mx_build_order(const Dev& d, const StepScalars* tab, int row, bool all,
                           cudaStream_t st) {
  k_mx_build_order<<<nblk(d.ntot, kOrderWindow), kOrderWindow, 0, st>>>(d, tab, row,
                                                                         all ? 1 : 0);
}

void launch_pass_mixed(const Dev& d, int mode, bool se, const StepScalars* tab, int row,
                       cudaStream_t st, int block) {
  if (block <= 0) block = 128;
  if (d.pass_kind == 1) {
    switch (mode) {
      case PASS_FORCE: launch_tile<PASS_FORCE>(d, tab, row, st); break;
      case PASS_CORR_STRAIN: launch_tile<PASS_CORR_STRAIN>(d, tab, row, st); break;
      case PASS_PRED_STRAIN: launch_tile<PASS_PRED_STRAIN>(d, tab, row, st); break;
      case PASS_CORR_RESIZE: launch_tile<PASS_CORR_RESIZE>(d, tab, row, st); break;
      case PASS_PRED_RESIZE: launch_tile<PASS_PRED_RESIZE>(d, tab, row, st); break;
    }
  } else {
    switch (mode) {
      case PASS_FORCE: launch_one<PASS_FORCE>(d, tab, row, st, block); break;
      case PASS_CORR_STRAIN: launch_one<PASS_CORR_STRAIN>(d, tab, row, st, block); break;
      case PASS_PRED_STRAIN: launch_one<PASS_PRED_STRAIN>(d, tab, row, st, block); break;
      case PASS_CORR_RESIZE: launch_one<PASS_CORR_RESIZE>(d, tab, row, st, block); break;
      case PASS_PRED_RESIZE: launch_one<PASS_PRED_RESIZE>(d, tab, row, st, block); break;
    }
  }
  // stress and energy of the state (forces and predictor passes) in FP64
  if (se) launch_mx_se64(d, tab, row, st);
}

bool launch_persist_steps(const Dev& d, const StepScalars* tab, int row0, int nsteps, int* out,
                          cudaStream_t st) {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return false;
  const void* fn = d.contact_model == 1 ? (const void*)k_persist_steps<true>
                                        : (const void*)k_persist_steps<false>;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 128, 0) != cudaSuccess ||
      per_sm < 1)
    return false;
  int grid = sms * per_sm;
  const int need = (d.ntot + 127) / 128;
  if (need < grid) grid = need;
  Dev dd = d;
  dd.cond = 0;  // no graph node to switch: the launch ends at a pending rebuild
  void* args[] = {&dd, (void*)&tab, &row0, &nsteps, &out};
  return cudaLaunchCooperativeKernel(fn, grid, 128, args, 0, st) == cudaSuccess;
}

bool launch_persist_fire(const Dev& d, const FireState& f, const StepScalars* tab, double ftol,
                         double dt_max, int iters, int* out, cudaStream_t st) {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return false;
  const void* fn = d.contact_model == 1 ? (const void*)k_persist_fire<true>
                                        : (const void*)k_persist_fire<false>;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, 0) != cudaSuccess ||
      per_sm < 1)
    return false;
  int grid = sms * per_sm;
  const int need = (d.ntot + 255) / 256;
  if (need < grid) grid = need;
  Dev dd = d;
  dd.cond = 0;
  dd.skip = f.done;  // converged systems: no force pass
  FireState ff = f;
  void* args[] = {&dd, &ff, (void*)&tab, &ftol, &dt_max, &iters, &out};
  return cudaLaunchCooperativeKernel(fn, grid, 256, args, 0, st) == cudaSuccess;
}

void launch_tile_lists(const Dev& d, bool all, cudaStream_t st) {
  k_tile_lists<<<d.ntiles, kTileThreads, 0, st>>>(d, all ? 1 : 0);
}

void launch_mx_materialize(const Dev& d, const StepScalars* tab, int row, bool all,
                           cudaStream_t st) {
  if (all)
    k_mx_materialize<<<nblk(d.ntot, 256), 256, 0, st>>>(d, tab, row, 1);
  else
    k_mx_materialize<<<kWalkBlocks, 256, 0, st>>>(d, tab, row, 0);
}

void launch_mx_local(const Dev& d, const StepScalars* tab, int row, bool all, cudaStream_t st) {
  k_mx_local<<<kWalkBlocks, 256, 0, st>>>(d, tab, row, all ? 1 : 0);
}

void launch_mx_build_list(const Dev& d, const StepScalars* tab, int row, bool all,
                          cudaStream_t st) {
  k_mx_build_list<<<2 * kWalkBlocks, 128, 0, st>>>(d, tab, row, all ? 1 : 0);
}

}  // namespace sc
