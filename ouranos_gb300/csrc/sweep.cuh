// Transport sweep kernel for sm_103a.
//
// Replaces the reference's task loop
//   initialize_scheduler(); while (n_tasks_to_execute) sweep(*get_next_task(), ...)
// (src/RadiativeTransfer.cc:605-692, 780-809, 878-1012), whose scheduler walks a
// (cell, direction) task DAG with FIFO ready counters and MPI face messages.
//
// Canonical orientation.  A direction with Omega_a < 0 is swept in the mirrored
// coordinate x'_a = N_a - 1 - x_a, and each cell's local dofs are visited in the
// mirrored order, so every direction looks like one of the all-positive octant:
// the inflow face of axis a is local index c_a = 0 and the outflow face
// c_a = p.  Face dof positions are then compile-time constants and the cell
// matrix depends only on (sigma_t, |Omega|) (its inverse is precomputed).
//
// Work decomposition.  The sweep axis S is y in 2-D and z in 3-D; the
// transverse plane (x, or x-y) is cut into tiles of wx (x wy) cells.  One warp
// runs one task = (group of kd directions of one octant, one tile): lane
// (lx, ly, k) handles cell (x'_0 + lx, y'_0 + ly) of direction k and, at step
// s, the plane s' = s - lx - ly of the sweep axis (a skewed wavefront inside
// the warp).  Upwind face values arrive
//   - along S: from the lane's own previous step (registers),
//   - along x/y inside the tile: from lane-1 / lane-wx by warp shuffle,
//   - across tiles: from an HBM edge buffer written by the upwind tile's warp,
//     guarded by a per-(group, tile) progress counter (release store /
//     acquire load) -- the GPU form of the reference's MPI_Isend/Iprobe of
//     outflow faces (src/RadiativeTransfer.cc:633-750).
// Tasks are handed out through one atomic ticket in dependency order (tile
// level first), so a warp only ever waits on tasks that live warps already
// hold: any grid size is deadlock-free.  Every wait is bounded (iteration cap
// and %globaltimer); a wait that runs out sets `status`, and all warps leave.
//
// Per lane and step: b = q_d[cell] (the source expanded to this direction by
// the expansion kernel, or sum_m M2D(d,m) T_m[cell] + isotropic source for one
// or two moments) + |Omega_a| F_a psi_up,a over the inflow faces; x = A'^-1 b;
// the outflow faces are the c_a = p entries of x; x is stored as psi_d[cell].
// The next step's source values are loaded one step ahead, so their memory
// latency overlaps the current solve.  The moments phi = D2M psi are formed
// afterwards by the reduction kernel over the direction axis (no atomics: the
// sweep is deterministic).
#pragma once

#include "internal.h"

namespace ouranos {

__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_gpu(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ long long global_ns() {
  long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Wait until *flag >= target.  Returns false when the wait ran out (and then
// records status 1) or when another warp has already recorded an error.
static __device__ __forceinline__ bool wait_at_least(const int* flag, int target, int* status,
                                                     long long limit_ns) {
  if (ld_acquire_gpu(flag) >= target) return true;
  const long long t0 = global_ns();
  unsigned sleep_ns = 32;
  for (unsigned it = 0; it < (1u << 26); ++it) {
    if (ld_acquire_gpu(flag) >= target) return true;
    if (*(volatile int*)status) return false;
    if (global_ns() - t0 > limit_ns) break;
    __nanosleep(sleep_ns);
    if (sleep_ns < 512) sleep_ns <<= 1;
  }
  atomicCAS(status, 0, 1);
  return false;
}

template <int DIM, int P1>
struct Cell {
  static constexpr int N = DIM == 2 ? P1 * P1 : P1 * P1 * P1;
  static constexpr int FD = DIM == 2 ? P1 : P1 * P1;
  static constexpr int PN = N / P1;  // dofs per sweep-axis layer
  // canonical local component of dof i on axis a
  static __device__ __forceinline__ constexpr int comp(int i, int a) {
    return a == 0 ? i % P1 : (a == 1 ? (i / P1) % P1 : i / (P1 * P1));
  }
  // dof on the inflow (c_a = 0) face of the x axis, transverse index t
  static __device__ __forceinline__ constexpr int x_in(int t) { return P1 * t; }
  static __device__ __forceinline__ constexpr int x_out(int t) { return P1 * t + P1 - 1; }
  // y axis (3-D only), transverse t = c_x + P1 c_z
  static __device__ __forceinline__ constexpr int y_in(int t) { return (t % P1) + P1 * P1 * (t / P1); }
  static __device__ __forceinline__ constexpr int y_out(int t) { return y_in(t) + P1 * (P1 - 1); }
  // sweep axis (y in 2-D, z in 3-D)
  static __device__ __forceinline__ constexpr int s_in(int t) { return t; }
  static __device__ __forceinline__ constexpr int s_out(int t) { return t + N - PN; }
};

template <typename real, int DIM, int P1, int FM>
__global__ void __launch_bounds__(128) sweep_kernel(const SweepArgs<real> a) {
  using C = Cell<DIM, P1>;
  constexpr int N = C::N;
  constexpr int FD = C::FD;
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int wc = a.wx * a.wy;
  const int kslot = lane / wc;
  const int cl = lane - kslot * wc;
  const int lx = cl % a.wx;
  const int ly = cl / a.wx;
  const int tiles = a.tiles_x * a.tiles_y;
  const int NS = a.n_sweep;
  const int NX = a.nx;
  const int NY = DIM == 3 ? a.ny : 1;
  const int nsteps = NS + (a.wx - 1) + (a.wy - 1);
  constexpr int AS = DIM - 1;  // physical axis of the sweep direction

  for (;;) {
    int task = 0, stop = 0;
    if (lane == 0) {
      task = atomicAdd(a.ticket, 1);
      stop = *(volatile int*)a.status;
    }
    task = __shfl_sync(FULL, task, 0);
    stop = __shfl_sync(FULL, stop, 0);
    if (task >= a.n_tasks || stop) return;

    const int2 tk = a.tasks[task];
    const int grp = tk.x, tile = tk.y;
    const int tx = tile % a.tiles_x, ty = tile / a.tiles_x;
    const int d = a.group_dirs[grp * a.kd + kslot];
    const bool dir_ok = d >= 0;
    const int dd = dir_ok ? d : 0;
    const int flip = a.group_flip[grp];
    const real wX = a.abs_omega[dd * 3 + 0];
    const real wY = DIM == 3 ? a.abs_omega[dd * 3 + 1] : real(0);
    const real wS = a.abs_omega[dd * 3 + AS];
    real bX = 0, bY = 0, bS = 0;
    if (a.bnd) {
      bX = a.bnd[dd * 3 + 0];
      if (DIM == 3) bY = a.bnd[dd * 3 + 1];
      bS = a.bnd[dd * 3 + AS];
    }
    real w0 = 0, w1 = 0;  // M2D row (moment-fused form)
    if (FM >= 1) w0 = a.m2d[(size_t)dd * a.n_mom + 0];
    if (FM >= 2) w1 = a.m2d[(size_t)dd * a.n_mom + 1];
    const int dcls = a.dir_class[dd];
    // mirrored local dof offsets: phys(i') = base + c0*s0 + c1*s1 + c2*s2
    int base = 0, st0 = 1, st1 = P1, st2 = P1 * P1;
    if (flip & 1) { base += (P1 - 1); st0 = -1; }
    if (flip & 2) { base += (P1 - 1) * P1; st1 = -P1; }
    if (DIM == 3 && (flip & 4)) { base += (P1 - 1) * P1 * P1; st2 = -P1 * P1; }

    const int xc = tx * a.wx + lx;  // canonical transverse coordinates
    const int yc = ty * a.wy + ly;
    const bool col_ok = dir_ok && xc < NX && (DIM == 2 || yc < NY);
    const int xp = (flip & 1) ? NX - 1 - xc : xc;  // physical
    const int yp = DIM == 3 ? ((flip & 2) ? NY - 1 - yc : yc) : 0;
    const int sflip = DIM == 3 ? (flip & 4) : (flip & 2);
    const long colbase = DIM == 2 ? (long)xp : (long)xp + (long)NX * yp;
    const long plane = DIM == 2 ? (long)NX : (long)NX * NY;  // cells per sweep-axis layer
    auto cell_of = [&](int sc) { return colbase + plane * (sflip ? NS - 1 - sc : sc); };
    const size_t dirbase = (size_t)dd * a.n_dofs;

    const int* prog_x = a.progress + grp * tiles + tile - 1;
    const int* prog_y = a.progress + grp * tiles + tile - a.tiles_x;
    int* prog_self = a.progress + grp * tiles + tile;
    const bool pub_x = tx + 1 < a.tiles_x;
    const bool pub_y = DIM == 3 && ty + 1 < a.tiles_y;
    const bool publish = pub_x || pub_y;

    // source values of the lane's next cell, loaded one step ahead
    real nq[N], nt1[FM >= 2 ? N : 1], niso[FM >= 1 ? N : 1];
    int ncls = 0;
    auto load_next = [&](int sc) {
      const long cb = cell_of(sc) * N + base;
      ncls = __ldg(a.cell_class + cell_of(sc));
      if (FM == 0) {
        const real* Q = a.q + dirbase + cb;
#pragma unroll
        for (int i = 0; i < N; ++i)
          nq[i] = __ldg(Q + C::comp(i, 0) * st0 + C::comp(i, 1) * st1 + (DIM == 3 ? C::comp(i, 2) * st2 : 0));
      } else {
        const real* T = a.src + cb;
#pragma unroll
        for (int i = 0; i < N; ++i) {
          const int off = C::comp(i, 0) * st0 + C::comp(i, 1) * st1 + (DIM == 3 ? C::comp(i, 2) * st2 : 0);
          nq[i] = __ldg(T + off);
          if (FM >= 2) nt1[i] = __ldg(T + a.n_dofs + off);
          if (FM >= 1) niso[i] = a.iso ? __ldg(a.iso + cb + off) : real(0);
        }
      }
    };
    // the lane's first active step is s = lx + ly (plane 0)
    if (col_ok) load_next(0);

    real psiS[FD], psiX[FD], psiY[FD];
#pragma unroll
    for (int t = 0; t < FD; ++t) psiS[t] = psiX[t] = psiY[t] = real(0);

    for (int s = 0; s < nsteps; ++s) {
      const int sc = s - lx - ly;
      const bool act = col_ok && sc >= 0 && sc < NS;

      // ---- upwind face values.  Edge-buffer waits run first (divergent), the
      // shuffles after them (converged), and the boundary / edge / neighbour
      // choice is a branch-free select.
      real eX[FD], eY[FD];
#pragma unroll
      for (int t = 0; t < FD; ++t) eX[t] = eY[t] = real(0);
      bool failed = false;
      const bool need_x = act && lx == 0 && tx > 0;
      const bool need_y = DIM == 3 && act && ly == 0 && ty > 0;
      if (need_x) {
        if (wait_at_least(prog_x, sc + a.wx + ly + a.wait_bias, a.status, a.wait_limit_ns)) {
          const real* e = a.edge_x + ((((size_t)d * tiles + tile - 1) * NS + sc) * a.wy + ly) * FD;
#pragma unroll
          for (int t = 0; t < FD; ++t) eX[t] = e[t];
        } else {
          failed = true;
        }
      }
      if (need_y) {
        if (wait_at_least(prog_y, sc + lx + a.wy + a.wait_bias, a.status, a.wait_limit_ns)) {
          const real* e =
              a.edge_y + ((((size_t)d * tiles + tile - a.tiles_x) * NS + sc) * a.wx + lx) * FD;
#pragma unroll
          for (int t = 0; t < FD; ++t) eY[t] = e[t];
        } else {
          failed = true;
        }
      }
      if (__any_sync(FULL, failed)) break;  // status is set; every warp drains
      const bool x_edge = lx == 0;
      const bool y_edge = ly == 0;
      real upX[FD], upY[FD], upS[FD];
#pragma unroll
      for (int t = 0; t < FD; ++t) {
        const real sx = __shfl_up_sync(FULL, psiX[t], 1);
        upX[t] = x_edge ? (tx == 0 ? bX : eX[t]) : sx;
        if (DIM == 3) {
          const real sy = __shfl_up_sync(FULL, psiY[t], a.wx);
          upY[t] = y_edge ? (ty == 0 ? bY : eY[t]) : sy;
        }
        upS[t] = sc == 0 ? bS : psiS[t];
      }

      if (act) {
        const long cell = cell_of(sc);
        const long cbase = cell * N + base;
        const int cls = ncls;
        real b[N];
#pragma unroll
        for (int i = 0; i < N; ++i) {
          if (FM == 0) b[i] = nq[i];
          else if (FM == 1) b[i] = w0 * nq[i] + niso[i];
          else b[i] = w0 * nq[i] + w1 * nt1[i] + niso[i];
        }
        // prefetch the next plane's source while this one is solved
        if (sc + 1 < NS) load_next(sc + 1);
        // inflow faces: b_face += |Omega_a| F_a psi_up
        const real* FX = a.face_mass + 0 * FD * FD;
        const real* FS = a.face_mass + AS * FD * FD;
#pragma unroll
        for (int t = 0; t < FD; ++t) {
          real accx = 0, accs = 0;
#pragma unroll
          for (int u = 0; u < FD; ++u) {
            accx += __ldg(FX + t * FD + u) * upX[u];
            accs += __ldg(FS + t * FD + u) * upS[u];
          }
          b[C::x_in(t)] += wX * accx;
          b[C::s_in(t)] += wS * accs;
        }
        if (DIM == 3) {
          const real* FY = a.face_mass + 1 * FD * FD;
#pragma unroll
          for (int t = 0; t < FD; ++t) {
            real acc = 0;
#pragma unroll
            for (int u = 0; u < FD; ++u) acc += __ldg(FY + t * FD + u) * upY[u];
            b[C::y_in(t)] += wY * acc;
          }
        }
        // x = A'^-1 b
        const real* Ai = a.ainv + ((size_t)cls * a.n_dir_class + dcls) * (N * N);
        real x[N];
#pragma unroll
        for (int i = 0; i < N; ++i) {
          real acc = 0;
#pragma unroll
          for (int j = 0; j < N; ++j) acc += __ldg(Ai + i * N + j) * b[j];
          x[i] = acc;
        }
        real* P = a.psi + dirbase + cbase;
#pragma unroll
        for (int i = 0; i < N; ++i)
          P[C::comp(i, 0) * st0 + C::comp(i, 1) * st1 + (DIM == 3 ? C::comp(i, 2) * st2 : 0)] = x[i];
#pragma unroll
        for (int t = 0; t < FD; ++t) {
          psiX[t] = x[C::x_out(t)];
          psiS[t] = x[C::s_out(t)];
          if (DIM == 3) psiY[t] = x[C::y_out(t)];
        }
        if (lx == a.wx - 1 && pub_x) {
          real* e = a.edge_x + ((((size_t)d * tiles + tile) * NS + sc) * a.wy + ly) * FD;
#pragma unroll
          for (int t = 0; t < FD; ++t) e[t] = psiX[t];
        }
        if (DIM == 3 && ly == a.wy - 1 && pub_y) {
          real* e = a.edge_y + ((((size_t)d * tiles + tile) * NS + sc) * a.wx + lx) * FD;
#pragma unroll
          for (int t = 0; t < FD; ++t) e[t] = psiY[t];
        }
      }
      if (publish) {
        __threadfence();
        __syncwarp();
        if (lane == 0) st_release_gpu(prog_self, s + 1);
      }
    }
  }
}

template <typename real, int DIM, int P1>
cudaError_t launch_sweep_impl(int fm, const SweepArgs<real>& a, int grid, int block,
                              cudaStream_t s) {
  if (fm == 0)
    sweep_kernel<real, DIM, P1, 0><<<grid, block, 0, s>>>(a);
  else if (fm == 1)
    sweep_kernel<real, DIM, P1, 1><<<grid, block, 0, s>>>(a);
  else if (fm == 2)
    sweep_kernel<real, DIM, P1, 2><<<grid, block, 0, s>>>(a);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

}  // namespace ouranos
