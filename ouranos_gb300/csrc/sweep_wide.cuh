// One warp per cell: the transport sweep for cells whose dofs do not fit the
// per-lane register form of sweep.cuh (2-D Q5, 3-D Q3..Q5 -- the orders the
// reference dispatches in src/ouranos.cc:307-346, 397-436), and, as the
// 1 x 1 x 1 tiling, for every order.
//
// A task is one transverse column of one direction (wx = wy = kd = 1), swept
// cell by cell along the sweep axis; the 32 lanes of the warp share each cell
// solve.  Per step:
//   - the upwind faces of the neighbouring columns arrive through the same
//     tagged edge words as in the register form, one value per lane, each
//     polled with a bounded wait; the sweep-axis face is the previous step's
//     outflow, kept in the warp's shared-memory slot;
//   - lane l assembles the right-hand side rows i = l + 32 k (b = q_d[cell],
//     then the x, sweep-axis and y inflow faces in that order, the order of the
//     register form, so both forms round every dof the same way);
//   - x = A'^-1 b: lane l computes rows l + 32 k from the transposed inverse
//     table [class][|Omega| class][j][i], so the warp reads each table row j
//     as consecutive values, and b[j] is a shared-memory broadcast;
//   - the outflow faces are published first (the downwind columns wait on
//     them), then the cell's angular flux is stored.
// The source of the next cell is loaded one step ahead into registers.
// Tickets hand the columns out in dependency order (build_schedule), so the
// deadlock-freedom argument of the register form holds unchanged.
#pragma once

#include "sweep.cuh"

namespace ouranos {

// Shared-memory slot of one warp: b[N], x[N], and the three inflow faces
template <typename real, int DIM, int P1>
struct WideSlot {
  static constexpr int N = Cell<DIM, P1>::N;
  static constexpr int FD = Cell<DIM, P1>::FD;
  static constexpr size_t bytes = ((size_t)(2 * N + 3 * FD) * sizeof(real) + 15) & ~(size_t)15;
};

// dot product of table row `row` (FD values) with the face values in shared memory
template <typename real, int FD>
__device__ __forceinline__ real face_dot(const real* row, const real* up) {
  using A = Arith<real>;
  typename A::acc acc = A::prod(A::ldg(row), up[0]);
#pragma unroll 4
  for (int u = 1; u < FD; ++u) A::fma(acc, A::ldg(row + u), up[u]);
  return A::raw(acc);
}

template <typename real, int DIM, int P1>
__device__ __forceinline__ void sweep_wide_task(const SweepArgs<real>& a, const int task,
                                                unsigned char* smem_raw) {
  using C = Cell<DIM, P1>;
  using A = Arith<real>;
  constexpr int N = C::N;
  constexpr int FD = C::FD;
  constexpr int FDP = pad4(FD);
  constexpr int W = Tagged<real>::W;
  constexpr int NL = (N + 31) / 32;  // rows per lane
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int AS = DIM - 1;  // physical axis of the sweep direction
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  real* sb = reinterpret_cast<real*>(smem_raw + warp * WideSlot<real, DIM, P1>::bytes);
  real* sx = sb + N;
  real* sX = sx + N;
  real* sY = sX + FD;
  real* sS = sY + FD;

  const int tiles = a.tiles_x * a.tiles_y;
  const int NS = a.n_sweep;
  const int NX = a.nx;
  const int NY = DIM == 3 ? a.ny : 1;
  const unsigned want_epoch = a.epoch ^ (a.wait_bias ? 0x8000u : 0u);
  const int2 tk = a.tasks[task];
  const int grp = tk.x, tile = tk.y;
  const int tx = tile % a.tiles_x, ty = tile / a.tiles_x;
  const int d = a.group_dirs[grp];  // one direction per group
  if (d < 0) return;
  const int flip = a.group_flip[grp];
  const real wX = a.abs_omega[d * 3 + 0];
  const real wY = DIM == 3 ? a.abs_omega[d * 3 + 1] : real(0);
  const real wS = a.abs_omega[d * 3 + AS];
  real bX = 0, bY = 0, bS = 0;
  if (a.bnd) {
    bX = a.bnd[d * 3 + 0];
    if (DIM == 3) bY = a.bnd[d * 3 + 1];
    bS = a.bnd[d * 3 + AS];
  }
  const int dcls = a.dir_class[d];
  // mirrored local dof offsets: phys(i') = base + c0*s0 + c1*s1 + c2*s2
  int base = 0, st0 = 1, st1 = P1, st2 = P1 * P1;
  if (flip & 1) { base += (P1 - 1); st0 = -1; }
  if (flip & 2) { base += (P1 - 1) * P1; st1 = -P1; }
  if (DIM == 3 && (flip & 4)) { base += (P1 - 1) * P1 * P1; st2 = -P1 * P1; }
  int offs[NL];  // physical offset of this lane's rows within the cell
#pragma unroll
  for (int k = 0; k < NL; ++k) {
    const int i = lane + 32 * k;
    offs[k] = i < N ? base + C::comp(i, 0) * st0 + C::comp(i, 1) * st1 +
                          (DIM == 3 ? C::comp(i, 2) * st2 : 0)
                    : 0;
  }
  const int xp = (flip & 1) ? NX - 1 - tx : tx;  // physical column
  const int yp = DIM == 3 ? ((flip & 2) ? NY - 1 - ty : ty) : 0;
  const int sflip = DIM == 3 ? (flip & 4) : (flip & 2);
  const long colbase = DIM == 2 ? (long)xp : (long)xp + (long)NX * yp;
  const long plane = DIM == 2 ? (long)NX : (long)NX * NY;
  auto cell_of = [&](int sc) { return colbase + plane * (sflip ? NS - 1 - sc : sc); };
  const size_t dirbase = (size_t)d * a.n_dofs;
  const bool pub_x = tx + 1 < a.tiles_x;
  const bool pub_y = DIM == 3 && ty + 1 < a.tiles_y;
  auto edge_x_at = [&](int t, int r) {  // words of column tile t, plane r
    return a.edge_x + (((size_t)d * tiles + t) * NS + r) * (FD * W);
  };
  auto edge_y_at = [&](int t, int r) {
    return a.edge_y + (((size_t)d * tiles + t) * NS + r) * (FD * W);
  };
  const real* FX = a.face_mass + 0 * FD * FDP;
  const real* FYm = a.face_mass + 1 * FD * FDP;
  const real* FS = a.face_mass + AS * FD * FDP;

  for (int t = lane; t < FD; t += 32) sS[t] = bS;
  real qn[NL];
  auto load_q = [&](int sc) {
    const real* Q = a.q + dirbase + cell_of(sc) * N;
#pragma unroll
    for (int k = 0; k < NL; ++k)
      if (lane + 32 * k < N) qn[k] = A::ldg(Q + offs[k]);
  };
  load_q(0);
  int cls_n = __ldg(a.cell_class + cell_of(0));

  for (int sc = 0; sc < NS; ++sc) {
    real qc[NL];
#pragma unroll
    for (int k = 0; k < NL; ++k) qc[k] = qn[k];
    const int cls = cls_n;
    if (sc + 1 < NS) {  // the next cell's source and class, one step ahead
      load_q(sc + 1);
      cls_n = __ldg(a.cell_class + cell_of(sc + 1));
    }
    // ---- upwind faces of the neighbouring columns (or the boundary)
    const unsigned tag = (want_epoch << 16) | ((unsigned)sc & 0xffffu);
    bool failed = false;
    for (int t = lane; t < FD; t += 32) {
      real v = bX;
      if (tx > 0) failed |= !fetch_edge<real, 1>(edge_x_at(tile - 1, sc) + t * W, tag, &v, a.status, a.wait_limit_ns);
      sX[t] = v;
      if (DIM == 3) {
        real w = bY;
        if (ty > 0)
          failed |= !fetch_edge<real, 1>(edge_y_at(tile - a.tiles_x, sc) + t * W, tag, &w, a.status, a.wait_limit_ns);
        sY[t] = w;
      }
    }
    if (__any_sync(FULL, failed)) return;  // status is set; the kernel loop leaves
    __syncwarp();
    // ---- right-hand side: q, then |Omega_a| F_a psi_up on the inflow faces
#pragma unroll
    for (int k = 0; k < NL; ++k) {
      const int i = lane + 32 * k;
      if (i < N) {
        real bi = qc[k];
        if (C::comp(i, 0) == 0) {  // x inflow face, transverse index i / P1
          typename A::acc bx = A::from(bi);
          A::fma(bx, wX, face_dot<real, FD>(FX + (i / P1) * FDP, sX));
          bi = A::raw(bx);
        }
        if (C::comp(i, AS) == 0) {  // sweep-axis inflow face, transverse index i
          typename A::acc bs = A::from(bi);
          A::fma(bs, wS, face_dot<real, FD>(FS + i * FDP, sS));
          bi = A::raw(bs);
        }
        if (DIM == 3 && C::comp(i, 1) == 0) {  // y inflow face, transverse c_x + P1 c_z
          typename A::acc by = A::from(bi);
          A::fma(by, wY, face_dot<real, FD>(FYm + ((i % P1) + P1 * (i / (P1 * P1))) * FDP, sY));
          bi = A::raw(by);
        }
        sb[i] = bi;
      }
    }
    __syncwarp();
    // ---- x = A'^-1 b, rows lane + 32 k, ascending j
    const real* AT = a.ainv + ((size_t)cls * a.n_dir_class + dcls) * (size_t)(N * N);
    typename A::acc acc[NL];
    {
      const real b0 = sb[0];
#pragma unroll
      for (int k = 0; k < NL; ++k) acc[k] = lane + 32 * k < N ? A::prod(A::ldg(AT + lane + 32 * k), b0) : A::zero();
    }
#pragma unroll 4
    for (int j = 1; j < N; ++j) {
      const real bj = sb[j];
      const real* col = AT + (size_t)j * N + lane;
#pragma unroll
      for (int k = 0; k < NL; ++k)
        if (lane + 32 * k < N) A::fma(acc[k], A::ldg(col + 32 * k), bj);
    }
    real xv[NL];
#pragma unroll
    for (int k = 0; k < NL; ++k) {
      xv[k] = A::get(acc[k]);
      if (lane + 32 * k < N) sx[lane + 32 * k] = xv[k];
    }
    __syncwarp();
    // ---- outflow faces first (the downwind columns wait on them), then psi
    const unsigned ptag = (a.epoch << 16) | ((unsigned)sc & 0xffffu);
    for (int t = lane; t < FD; t += 32) {
      if (pub_x) Tagged<real>::put(edge_x_at(tile, sc) + t * W, sx[C::x_out(t)], ptag);
      if (pub_y) Tagged<real>::put(edge_y_at(tile, sc) + t * W, sx[C::y_out(t)], ptag);
      sS[t] = sx[C::s_out(t)];
    }
    real* P = a.psi + dirbase + cell_of(sc) * N;
#pragma unroll
    for (int k = 0; k < NL; ++k)
      if (lane + 32 * k < N) store_stream(P + offs[k], xv[k]);
    __syncwarp();  // sb / sx / sS are rewritten by the next step
  }
}

template <typename real, int DIM, int P1>
__global__ void __launch_bounds__(128) sweep_wide_kernel(const SweepArgs<real> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr unsigned FULL = 0xffffffffu;
  for (;;) {
    int task = 0, stop = 0;
    if ((threadIdx.x & 31) == 0) {
      task = atomicAdd(a.ticket, 1);
      stop = *(volatile int*)a.status;
    }
    task = __shfl_sync(FULL, task, 0);
    stop = __shfl_sync(FULL, stop, 0);
    if (task >= a.n_tasks || stop) return;
    sweep_wide_task<real, DIM, P1>(a, task, smem_raw);
  }
}

template <typename real, int DIM, int P1>
cudaError_t launch_sweep_wide_impl(const SweepArgs<real>& a, int grid, int block, cudaStream_t s) {
  const size_t smem = (size_t)(block / 32) * WideSlot<real, DIM, P1>::bytes;
  sweep_wide_kernel<real, DIM, P1><<<grid, block, smem, s>>>(a);
  return cudaGetLastError();
}

// every order of both dimensions (2-D and 3-D Q1..Q5)
template <typename real>
cudaError_t launch_sweep_wide_any(int dim, int p1, const SweepArgs<real>& a, int grid, int block,
                                  cudaStream_t s) {
  if (dim == 2) {
    switch (p1) {
      case 2: return launch_sweep_wide_impl<real, 2, 2>(a, grid, block, s);
      case 3: return launch_sweep_wide_impl<real, 2, 3>(a, grid, block, s);
      case 4: return launch_sweep_wide_impl<real, 2, 4>(a, grid, block, s);
      case 5: return launch_sweep_wide_impl<real, 2, 5>(a, grid, block, s);
      case 6: return launch_sweep_wide_impl<real, 2, 6>(a, grid, block, s);
    }
  } else if (dim == 3) {
    switch (p1) {
      case 2: return launch_sweep_wide_impl<real, 3, 2>(a, grid, block, s);
      case 3: return launch_sweep_wide_impl<real, 3, 3>(a, grid, block, s);
      case 4: return launch_sweep_wide_impl<real, 3, 4>(a, grid, block, s);
      case 5: return launch_sweep_wide_impl<real, 3, 5>(a, grid, block, s);
      case 6: return launch_sweep_wide_impl<real, 3, 6>(a, grid, block, s);
    }
  }
  return cudaErrorInvalidValue;
}

}  // namespace ouranos
