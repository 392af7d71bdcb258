// Temporal blocking on the GPU: K time steps per launch inside a shared-memory
// tile, for programs whose step is a single stage (every manifest value is a
// store).  This replaces the reference's CPU temporal blocking
// (Templates.hs:311-381: floor/wall buffers walked block by block): each
// CTA loads its output tile plus a halo of K*R cells (R: how far the stencil
// reads) with periodic wrap, advances K steps in shared memory, shrinking the
// valid region by R per step, and writes the tile rolled by K*shift.  The
// same generated stage functor runs per cell, so the result is bit-identical
// to K single steps of the generic kernel.
#pragma once
#include <string.h>
#include <utility>

#include "fgb_templates.cuh"
#include "fgb_wait.cuh"

namespace fgb {

// Accessor over a shared-memory tile: cursor loads read the current buffer,
// stores write the next one.  Layout [field][row][col], col contiguous.
template <class T, int NF, int RY, int RX>
struct TileAccess {
  const T* cur;
  T* nxt;
  int ly, lx;
  template <int F, int D0, int D1, int D2>
  __device__ __forceinline__ T ld() const {
    static_assert(D0 == 0, "2D tile");
    return cur[(F * RY + ly + D1) * RX + lx + D2];
  }
  template <int F>
  __device__ __forceinline__ void st(T v) const {
    nxt[(F * RY + ly) * RX + lx] = v;
  }
};

// Same tile, but stores go to registers: a thread computes several rows of
// one column before writing any of them, so loads shared between the rows
// (the vertical neighbours) are read from shared memory once.
template <class T, int NF, int RY, int RX>
struct RegTileAccess {
  const T* cur;
  T* res;
  int ly, lx;
  template <int F, int D0, int D1, int D2>
  __device__ __forceinline__ T ld() const {
    static_assert(D0 == 0, "2D tile");
    return cur[(F * RY + ly + D1) * RX + lx + D2];
  }
  template <int F>
  __device__ __forceinline__ void st(T v) const {
    res[F] = v;
  }
};

__device__ __forceinline__ int pmod(int a, int n) {
  int r = a % n;
  return r < 0 ? r + n : r;
}

// Periodic index for -n <= a < 2n (tile halos are shorter than the grid):
// a compare and an add instead of an integer division.
__device__ __forceinline__ int pwrap(int a, int n) {
  a += a < 0 ? n : 0;
  return a >= n ? a - n : a;
}

// TMA load of one tile (with halo) per field into shared memory: one
// elected thread arms an mbarrier with the expected bytes and issues one 2D
// box copy per field; every thread waits on the barrier for at most one
// second of the global timer.  Returns false (and raises the launch's error
// flag) if the wait ran out; the leader then waits once more, with the
// longer drain limit, so that a late copy lands before the block's shared
// memory is released.  The box lies inside the grid: the caller checks that.
template <class T, int NF, int PLANE>
__device__ __forceinline__ bool tma_load_tile(const FgbLaunch& L, T* smem, int x, int y) {
  __shared__ __align__(8) uint64_t bar;
  const uint32_t b = (uint32_t)__cvta_generic_to_shared(&bar);
  const bool leader = threadIdx.x == 0 && threadIdx.y == 0;
  if (leader) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (leader) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b),
                 "r"((uint32_t)(NF * PLANE * sizeof(T)))
                 : "memory");
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      const char* map = static_cast<const char*>(L.tmap) + f * FGB_TMA_MAP_BYTES;
      const uint32_t dst = (uint32_t)__cvta_generic_to_shared(smem + f * PLANE);
      asm volatile(
          "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
          "l"(map), "r"(x), "r"(y), "r"(b)
          : "memory");
    }
  }
  const bool ok = __syncthreads_and(mbar_wait_bounded(b, 0u));
  if (!ok && leader) {
    mbar_wait_bounded(b, 0u, kDrainLimitNs);
    if (L.err) atomicExch(L.err, 1);
  }
  return ok;
}

// K steps of a tile held in shared memory (two buffers of NF planes of
// RY x RX points).  Step k computes the region that is still exact after k+1
// steps, (k+1)R points in from the edge.  With RB > 1 a thread computes RB
// rows of a column into registers before storing any of them, so the
// vertical neighbours shared by those rows are read once.
template <class M, class Stage, class T, int NF, int R, int RY, int RX, int K, int BX, int BY, int RB>
__device__ __forceinline__ void tile_steps(T* smem, const typename M::U* __restrict__ U) {
  constexpr int PLANE = RY * RX;
#pragma unroll 1
  for (int k = 0; k < K; ++k) {
    const T* cur = smem + (k & 1) * NF * PLANE;
    T* nxt = smem + ((k + 1) & 1) * NF * PLANE;
    const int lo = (k + 1) * R;
    if constexpr (RB == 1) {
      for (int ly = lo + threadIdx.y; ly < RY - lo; ly += BY) {
        for (int lx = lo + threadIdx.x; lx < RX - lo; lx += BX) {
          TileAccess<T, NF, RY, RX> a{cur, nxt, ly, lx};
          eval<M, Stage>(a, U);
        }
      }
    } else {
      const int last = RY - lo - 1;   // rows past the region are clamped (computed, not stored)
      for (int ly0 = lo + threadIdx.y * RB; ly0 <= last; ly0 += BY * RB) {
        for (int lx = lo + threadIdx.x; lx < RX - lo; lx += BX) {
          T res[RB][NF];
#pragma unroll
          for (int r = 0; r < RB; ++r) {
            RegTileAccess<T, NF, RY, RX> a{cur, res[r], min(ly0 + r, last), lx};
            eval<M, Stage>(a, U);
          }
#pragma unroll
          for (int r = 0; r < RB; ++r) {
            if (ly0 + r <= last) {
#pragma unroll
              for (int f = 0; f < NF; ++f) nxt[(f * RY + ly0 + r) * RX + lx] = res[r][f];
            }
          }
        }
      }
    }
    __syncthreads();
  }
}

template <class M, class S, class Prog, class Stage, int TX, int TY, int K, int BX, int BY, int RB, bool TMA>
__global__ void __launch_bounds__(BX * BY) tb2d_kernel(const __grid_constant__ FgbLaunch L) {
  using T = typename M::T;
  constexpr int NF = Prog::kFields;
  constexpr int R = Prog::kReach;
  constexpr int H = K * R;
  constexpr int RY = TY + 2 * H, RX = TX + 2 * H;
  constexpr int PLANE = RY * RX;
  static_assert(Prog::kShift >= 0, "the per-step roll is non-negative");
  extern __shared__ __align__(16) unsigned char fgb_smem_raw[];
  // TMA writes to 128-byte aligned shared memory: the variant allocates 128
  // spare bytes and the tile starts at the next 128-byte boundary
  const uint32_t base = (uint32_t)__cvta_generic_to_shared(fgb_smem_raw);
  T* smem = reinterpret_cast<T*>(fgb_smem_raw + (TMA ? ((128u - (base & 127u)) & 127u) : 0u));
  const int ny = L.n[1], nx = L.n[2];
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const T* __restrict__ U = static_cast<const T*>(L.uniforms);

  // load the tile and its halo (periodic); halos shorter than the grid use
  // the cheap wrap.  Tiles whose halo lies inside the grid come by TMA.
  const bool small = TY + H >= ny || TX + H >= nx || K * Prog::kShift >= ny || K * Prog::kShift >= nx;
  bool loaded = false;
  if constexpr (TMA) {
    static_assert(RX == FGB_TMA_BOX && RY == FGB_TMA_BOX, "the tensor maps' box is the tile with its halo");
    static_assert(std::is_same<S, T>::value && (H * sizeof(T)) % 16 == 0 && (TX * sizeof(T)) % 16 == 0,
                  "box starts on a 16-byte boundary");
    if (L.tmap != nullptr && x0 >= H && y0 >= H && x0 + TX + H <= nx && y0 + TY + H <= ny) {
      if (!tma_load_tile<T, NF, PLANE>(L, smem, x0 - H, y0 - H)) return;
      loaded = true;
    }
  }
  if (!loaded) {
    for (int ly = threadIdx.y; ly < RY; ly += BY) {
      const int gy = small ? pmod(y0 - H + ly, ny) : pwrap(y0 - H + ly, ny);
      for (int lx = threadIdx.x; lx < RX; lx += BX) {
        const int gx = small ? pmod(x0 - H + lx, nx) : pwrap(x0 - H + lx, nx);
        const uint32_t g = (uint32_t)gy * (uint32_t)nx + (uint32_t)gx;
#pragma unroll
        for (int f = 0; f < NF; ++f)
          smem[f * PLANE + ly * RX + lx] = Storage<S, T>::load(static_cast<const S*>(L.in[f])[g], L.scale[f]);
      }
    }
    __syncthreads();
  }

  tile_steps<M, Stage, T, NF, R, RY, RX, K, BX, BY, RB>(smem, U);

  // store the tile, rolled by K steps' worth of shift
  const T* fin = smem + (K & 1) * NF * PLANE;
  for (int ty = threadIdx.y; ty < TY; ty += BY) {
    const int py = y0 + ty;
    if (py >= ny) break;
    const int oy = small ? (py + K * Prog::kShift) % ny : pwrap(py + K * Prog::kShift, ny);
    for (int tx = threadIdx.x; tx < TX; tx += BX) {
      const int px = x0 + tx;
      if (px >= nx) break;
      const int ox = small ? (px + K * Prog::kShift) % nx : pwrap(px + K * Prog::kShift, nx);
      const uint32_t g = (uint32_t)oy * (uint32_t)nx + (uint32_t)ox;
#pragma unroll
      for (int f = 0; f < NF; ++f)
        static_cast<S*>(L.out[f])[g] =
            Storage<S, T>::store(fin[f * PLANE + (ty + H) * RX + tx + H], L.inv_scale[f]);
    }
  }
}

template <class Prog, int P, class Stage, int TX, int TY, int K, int RB = 1, int BY_ = 8, bool TMA = false>
struct Tb2dVariant {
  using M = typename Precision<P>::M;
  using S = typename Precision<P>::S;
  using T = typename M::T;
  static constexpr int BX = 32, BY = BY_;
  static constexpr int H = K * Prog::kReach;
  static constexpr size_t kSmem =
      (size_t)2 * Prog::kFields * (TY + 2 * H) * (TX + 2 * H) * sizeof(T) + (TMA ? 128 : 0);

  static cudaError_t launch(const FgbLaunch* L, cudaStream_t stream) {
    auto kern = tb2d_kernel<M, S, Prog, Stage, TX, TY, K, BX, BY, RB, TMA>;
    static bool configured = false;
    if (!configured) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
      if (e != cudaSuccess) return e;
      configured = true;
    }
    dim3 grid((L->n[2] + TX - 1) / TX, (L->n[1] + TY - 1) / TY, 1);
    kern<<<grid, dim3(BX, BY), kSmem, stream>>>(*L);
    return cudaGetLastError();
  }
  static FgbFusedVariant describe() {
    FgbFusedVariant v;
    v.x_multiple = 1;
    v.launch = &launch;
    v.tile_x = TX;
    v.tile_y = TY;
    v.steps = K;
    v.smem_bytes = kSmem;
    return v;
  }
};

// Batched ensemble: persistent CTAs walk a queue of tiles drawn from every
// grid of the batch; each tile advances K steps in shared memory exactly like
// tb2d_kernel, with that grid's extent, periodic wrap and uniform table.
template <class M, class S, class Prog, class Stage, int TX, int TY, int K, int BX, int BY, int RB>
__global__ void __launch_bounds__(BX * BY) tb2d_batch_kernel(const __grid_constant__ FgbBatchLaunch B) {
  using T = typename M::T;
  constexpr int NF = Prog::kFields;
  constexpr int R = Prog::kReach;
  constexpr int H = K * R;
  constexpr int RY = TY + 2 * H, RX = TX + 2 * H;
  constexpr int PLANE = RY * RX;
  extern __shared__ __align__(16) unsigned char fgb_smem_raw[];
  T* smem = reinterpret_cast<T*>(fgb_smem_raw);
  for (int t = blockIdx.x; t < B.ntiles; t += gridDim.x) {
    const FgbBatchTile tile = B.tiles[t];
    const FgbBatchInstance in = B.inst[tile.inst];
    const int ny = in.ny, nx = in.nx;
    const size_t cells = (size_t)ny * nx;
    const S* src = static_cast<const S*>(in.state[B.parity]);
    S* dst = static_cast<S*>(in.state[B.parity ^ 1]);
    const T* __restrict__ U = static_cast<const T*>(in.uniforms);
    const int x0 = tile.x0, y0 = tile.y0;
    const bool small = TY + H >= ny || TX + H >= nx || K * Prog::kShift >= ny || K * Prog::kShift >= nx;
    for (int ly = threadIdx.y; ly < RY; ly += BY) {
      const int gy = small ? pmod(y0 - H + ly, ny) : pwrap(y0 - H + ly, ny);
      for (int lx = threadIdx.x; lx < RX; lx += BX) {
        const int gx = small ? pmod(x0 - H + lx, nx) : pwrap(x0 - H + lx, nx);
        const size_t g = (size_t)gy * nx + gx;
#pragma unroll
        for (int f = 0; f < NF; ++f)
          smem[f * PLANE + ly * RX + lx] = Storage<S, T>::load(src[f * cells + g], 1.0f);
      }
    }
    __syncthreads();
    tile_steps<M, Stage, T, NF, R, RY, RX, K, BX, BY, RB>(smem, U);
    const T* fin = smem + (K & 1) * NF * PLANE;
    for (int ty = threadIdx.y; ty < TY; ty += BY) {
      const int py = y0 + ty;
      if (py >= ny) break;
      const int oy = small ? (py + K * Prog::kShift) % ny : pwrap(py + K * Prog::kShift, ny);
      for (int tx = threadIdx.x; tx < TX; tx += BX) {
        const int px = x0 + tx;
        if (px >= nx) break;
        const int ox = small ? (px + K * Prog::kShift) % nx : pwrap(px + K * Prog::kShift, nx);
        const size_t g = (size_t)oy * nx + ox;
#pragma unroll
        for (int f = 0; f < NF; ++f)
          dst[f * cells + g] = Storage<S, T>::store(fin[f * PLANE + (ty + H) * RX + tx + H], 1.0f);
      }
    }
    __syncthreads();   // the next tile reuses the shared buffers
  }
}

template <class Prog, int P, class Stage, int TX, int TY, int K, int RB = 1, int BY_ = 8>
struct Tb2dBatchVariant {
  using M = typename Precision<P>::M;
  using S = typename Precision<P>::S;
  using T = typename M::T;
  static constexpr int BX = 32, BY = BY_;
  static constexpr int H = K * Prog::kReach;
  static constexpr size_t kSmem = (size_t)2 * Prog::kFields * (TY + 2 * H) * (TX + 2 * H) * sizeof(T);

  static cudaError_t configure() {
    static cudaError_t state = cudaErrorNotReady;
    if (state == cudaErrorNotReady)
      state = cudaFuncSetAttribute(tb2d_batch_kernel<M, S, Prog, Stage, TX, TY, K, BX, BY, RB>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
    return state;
  }
  static cudaError_t launch(const FgbBatchLaunch* B, cudaStream_t stream, int blocks) {
    cudaError_t e = configure();
    if (e != cudaSuccess) return e;
    tb2d_batch_kernel<M, S, Prog, Stage, TX, TY, K, BX, BY, RB><<<blocks, dim3(BX, BY), kSmem, stream>>>(*B);
    return cudaGetLastError();
  }
  static int blocks_per_sm() {
    if (configure() != cudaSuccess) return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, tb2d_batch_kernel<M, S, Prog, Stage, TX, TY, K, BX, BY, RB>,
                                                      BX * BY, kSmem) != cudaSuccess)
      return 0;
    return n;
  }
  static FgbBatchVariant describe() {
    FgbBatchVariant v;
    v.launch = &launch;
    v.blocks_per_sm = &blocks_per_sm;
    v.tile_x = TX;
    v.tile_y = TY;
    v.steps = K;
    v.smem_bytes = kSmem;
    return v;
  }
};

// 3D temporal blocking, 2.5D streaming: a CTA owns an x-y tile (plus a
// halo of K*R cells) and streams along the slowest axis.  For every level
// t = 0..K-1 it keeps a ring of 2R+1 planes in shared memory; each new input
// plane lets every level advance by one plane, and level K is written to
// HBM directly (rolled by K*shift).  Cursor loads along the streamed axis
// pick the ring slot, loads across it read the tile.
template <class T, int NF, int P, int RY, int RX>
struct PlaneAccess {
  const T* const* plane;  // the 2R+1 planes of the level below, z - R .. z + R
  int cell;               // ly * RX + lx
  T* res;
  template <int F, int D0, int D1, int D2>
  __device__ __forceinline__ T ld() const {
    return plane[D0 + P / 2][F * RY * RX + cell + D1 * RX + D2];
  }
  template <int F>
  __device__ __forceinline__ void st(T v) const {
    res[F] = v;
  }
};

__device__ __forceinline__ int ring_slot(int z, int p) {
  const int r = z % p;
  return r < 0 ? r + p : r;
}

// HX is the tile's halo in x and y: at least K*R, and wider where that puts
// the TMA box on a 16-byte boundary (the extra points are loaded and
// computed but never stored).
template <class M, class S, class Prog, class Stage, int TX, int TY, int K, int BX, int BY, bool TMA, int HX>
__global__ void __launch_bounds__(BX * BY) tb3d_kernel(const __grid_constant__ FgbLaunch L) {
  using T = typename M::T;
  constexpr int NF = Prog::kFields;
  constexpr int R = Prog::kReach;
  constexpr int H = K * R;                  // halo along the streamed axis
  static_assert(HX >= H, "the tile halo covers K steps");
  constexpr int P = 2 * R + 1;
  constexpr int D = TMA ? 2 : 0;            // input planes in flight ahead of the current one
  constexpr int P0 = P + D;                 // slots of the input ring
  constexpr int RY = TY + 2 * HX, RX = TX + 2 * HX;
  constexpr int PL = NF * RY * RX;          // one plane of every field
  static_assert(K >= 2, "the input ring is refilled after level 1 has read it");
  static_assert(Prog::kShift >= 0, "the per-step roll is non-negative");
  extern __shared__ __align__(16) unsigned char fgb_smem_raw[];
  // input ring [P0][NF][RY][RX], then the rings of levels 1..K-1 [P][NF][RY][RX];
  // TMA destinations start on 128-byte boundaries
  const uint32_t base = (uint32_t)__cvta_generic_to_shared(fgb_smem_raw);
  T* ring0 = reinterpret_cast<T*>(fgb_smem_raw + (TMA ? ((128u - (base & 127u)) & 127u) : 0u));
  const int nz = L.n[0], ny = L.n[1], nx = L.n[2];
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  // the streamed axis is cut into gridDim.z chunks of planes [z0, z1)
  const int zc = (nz + gridDim.z - 1) / gridDim.z;
  const int z0 = blockIdx.z * zc, z1 = min(nz, z0 + zc);
  if (z0 >= z1) return;
  const T* __restrict__ U = static_cast<const T*>(L.uniforms);
  const bool small = TY + HX >= ny || TX + HX >= nx || H >= nz || K * Prog::kShift >= nx ||
                     K * Prog::kShift >= ny || K * Prog::kShift >= nz;

  // Levels 1..K of input plane zin: level t works on plane zin - t*R from
  // the 2R+1 planes around it in the ring of level t-1.
  auto levels = [&](int zin) {
#pragma unroll 1
    for (int t = 1; t <= K; ++t) {
      const int zt = zin - t * R;
      if (zt < z0 - (K - t) * R) break;   // this level has nothing to compute yet
      const T* below = t == 1 ? ring0 : ring0 + (size_t)P0 * PL + (size_t)(t - 2) * P * PL;
      const int nslot = t == 1 ? P0 : P;
      const T* planes[P];
#pragma unroll
      for (int j = 0; j < P; ++j) planes[j] = below + ring_slot(zt - R + j, nslot) * PL;
      const int lo = t * R;
      if (t < K) {
        T* mine = ring0 + (size_t)P0 * PL + (size_t)(t - 1) * P * PL + ring_slot(zt, P) * PL;
        for (int ly = lo + threadIdx.y; ly < RY - lo; ly += BY) {
          for (int lx = lo + threadIdx.x; lx < RX - lo; lx += BX) {
            T res[NF];
            PlaneAccess<T, NF, P, RY, RX> a{planes, ly * RX + lx, res};
            eval<M, Stage>(a, U);
#pragma unroll
            for (int f = 0; f < NF; ++f) mine[(f * RY + ly) * RX + lx] = res[f];
          }
        }
        __syncthreads();
      } else {
        // final level: the tile's cells of plane zt, straight to HBM
        const int oz = small ? (zt + K * Prog::kShift) % nz : pwrap(zt + K * Prog::kShift, nz);
        for (int ty = threadIdx.y; ty < TY; ty += BY) {
          const int py = y0 + ty;
          if (py >= ny) break;
          const int oy = small ? (py + K * Prog::kShift) % ny : pwrap(py + K * Prog::kShift, ny);
          for (int tx = threadIdx.x; tx < TX; tx += BX) {
            const int px = x0 + tx;
            if (px >= nx) break;
            const int ox = small ? (px + K * Prog::kShift) % nx : pwrap(px + K * Prog::kShift, nx);
            T res[NF];
            PlaneAccess<T, NF, P, RY, RX> a{planes, (ty + HX) * RX + tx + HX, res};
            eval<M, Stage>(a, U);
            const size_t g = ((size_t)oz * ny + oy) * nx + ox;
#pragma unroll
            for (int f = 0; f < NF; ++f)
              static_cast<S*>(L.out[f])[g] = Storage<S, T>::store(res[f], L.inv_scale[f]);
          }
        }
      }
    }
  };
  const int zfirst = z0 - H, zend = z1 + H;   // input planes [zfirst, zend)

  if constexpr (TMA) {
    static_assert(RX == FGB_TMA_BOX && RY == FGB_TMA_BOX3_Y, "the tensor maps' box is one plane of the tile");
    static_assert(std::is_same<S, T>::value && (HX * sizeof(T)) % 16 == 0 && (TX * sizeof(T)) % 16 == 0,
                  "box starts on a 16-byte boundary");
    if (L.tmap != nullptr && x0 >= HX && y0 >= HX && x0 + TX + HX <= nx && y0 + TY + HX <= ny) {
      // Tiles whose halo is inside the grid in x and y stream their input
      // planes by TMA: plane z goes to ring slot z mod P0 and completes on
      // that slot's mbarrier; D planes are in flight ahead of the current one.
      __shared__ __align__(8) uint64_t bars[P0];
      const bool leader = threadIdx.x == 0 && threadIdx.y == 0;
      if (leader) {
#pragma unroll
        for (int j = 0; j < P0; ++j)
          asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"((uint32_t)__cvta_generic_to_shared(&bars[j]))
                       : "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      }
      __syncthreads();
      auto issue = [&](int z) {   // by the leader
        const int slot = ring_slot(z, P0);
        const int gz = small ? pmod(z, nz) : pwrap(z, nz);
        const uint32_t b = (uint32_t)__cvta_generic_to_shared(&bars[slot]);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b),
                     "r"((uint32_t)(PL * sizeof(T)))
                     : "memory");
#pragma unroll
        for (int f = 0; f < NF; ++f) {
          const char* map = static_cast<const char*>(L.tmap) + f * FGB_TMA_MAP_BYTES;
          const uint32_t dst = (uint32_t)__cvta_generic_to_shared(ring0 + slot * PL + f * RY * RX);
          asm volatile(
              "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
              "%4}], [%5];" ::"r"(dst),
              "l"(map), "r"(x0 - HX), "r"(y0 - HX), "r"(gz), "r"(b)
              : "memory");
        }
      };
      if (leader)
        for (int d = 0; d < D && zfirst + d < zend; ++d) issue(zfirst + d);
      for (int zin = zfirst; zin < zend; ++zin) {
        if (leader && zin + D < zend) issue(zin + D);
        // wait (bounded) for plane zin: the k-th use of a slot completes phase k
        const uint32_t b = (uint32_t)__cvta_generic_to_shared(&bars[ring_slot(zin, P0)]);
        const uint32_t parity = (uint32_t)((zin - zfirst) / P0) & 1u;
        if (!__syncthreads_and(mbar_wait_bounded(b, parity))) {
          if (leader) {
            // drain (bounded) the planes issued ahead before the block's
            // shared memory is released
            for (int z = zin; z <= zin + D && z < zend; ++z)
              mbar_wait_bounded((uint32_t)__cvta_generic_to_shared(&bars[ring_slot(z, P0)]),
                                (uint32_t)((z - zfirst) / P0) & 1u, kDrainLimitNs);
            if (L.err) atomicExch(L.err, 2);
          }
          return;
        }
        levels(zin);
        __syncthreads();
      }
      return;
    }
  }

  // Ordinary loads: the next input plane is fetched into registers while
  // the levels of the current one are computed, so its HBM latency is hidden.
  constexpr int NI = (RY + BY - 1) / BY, NJ = (RX + BX - 1) / BX;
  T pre[NI][NJ][NF];
  // the in-plane offsets of this thread's elements do not change from plane
  // to plane: wrap them once (-1 marks an element outside the tile)
  int yx[NI][NJ];
#pragma unroll
  for (int i = 0; i < NI; ++i) {
    const int ly = threadIdx.y + i * BY;
    const int gy = small ? pmod(y0 - HX + ly, ny) : pwrap(y0 - HX + ly, ny);
#pragma unroll
    for (int j = 0; j < NJ; ++j) {
      const int lx = threadIdx.x + j * BX;
      const int gx = small ? pmod(x0 - HX + lx, nx) : pwrap(x0 - HX + lx, nx);
      yx[i][j] = (ly < RY && lx < RX) ? gy * nx + gx : -1;
    }
  }
  const size_t plane_cells = (size_t)ny * nx;
  auto fetch = [&](int zin) {
    const size_t gz = (size_t)(small ? pmod(zin, nz) : pwrap(zin, nz)) * plane_cells;
#pragma unroll
    for (int i = 0; i < NI; ++i) {
#pragma unroll
      for (int j = 0; j < NJ; ++j) {
        if (yx[i][j] >= 0) {
          const size_t g = gz + (size_t)yx[i][j];
#pragma unroll
          for (int f = 0; f < NF; ++f)
            pre[i][j][f] = Storage<S, T>::load(static_cast<const S*>(L.in[f])[g], L.scale[f]);
        }
      }
    }
  };
  auto put = [&](int zin) {
    T* dst = ring0 + ring_slot(zin, P0) * PL + threadIdx.y * RX + threadIdx.x;
#pragma unroll
    for (int i = 0; i < NI; ++i) {
#pragma unroll
      for (int j = 0; j < NJ; ++j) {
        if (yx[i][j] >= 0) {
#pragma unroll
          for (int f = 0; f < NF; ++f) dst[f * RY * RX + i * BY * RX + j * BX] = pre[i][j][f];
        }
      }
    }
  };
  fetch(zfirst);
  put(zfirst);
  __syncthreads();
  for (int zin = zfirst; zin < zend; ++zin) {
    const bool more = zin + 1 < zend;
    if (more) fetch(zin + 1);
    levels(zin);
    // level 1 has read the ring slot that plane zin + 1 takes over
    if (more) put(zin + 1);
    __syncthreads();
  }
}

template <class Prog, int P, class Stage, int TX, int TY, int K, bool TMA = false, int HX = K * Prog::kReach>
struct Tb3dVariant {
  using M = typename Precision<P>::M;
  using S = typename Precision<P>::S;
  using T = typename M::T;
  static constexpr int BX = 32, BY = 8;
  static constexpr int H = K * Prog::kReach;
  static constexpr int Q = 2 * Prog::kReach + 1;   // slots per ring
  static constexpr size_t kSmem =
      (size_t)(K * Q + (TMA ? 2 : 0)) * Prog::kFields * (TY + 2 * HX) * (TX + 2 * HX) * sizeof(T) + (TMA ? 128 : 0);

  static cudaError_t launch(const FgbLaunch* L, cudaStream_t stream) {
    auto kern = tb3d_kernel<M, S, Prog, Stage, TX, TY, K, BX, BY, TMA, HX>;
    static bool configured = false;
    if (!configured) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
      if (e != cudaSuccess) return e;
      configured = true;
    }
    // enough CTAs to fill the SMs several times over; each chunk re-reads
    // 2H halo planes, so chunks stay at least 4H planes deep
    const int gx = (L->n[2] + TX - 1) / TX, gy = (L->n[1] + TY - 1) / TY;
    const int want = (1216 + gx * gy - 1) / (gx * gy);
    const int most = L->n[0] / (4 * H) > 1 ? L->n[0] / (4 * H) : 1;
    const int gz = want < most ? want : most;
    kern<<<dim3(gx, gy, gz), dim3(BX, BY), kSmem, stream>>>(*L);
    return cudaGetLastError();
  }
  static FgbFusedVariant describe() {
    FgbFusedVariant v;
    v.x_multiple = 1;
    v.launch = &launch;
    v.tile_x = TX;
    v.tile_y = TY;
    v.steps = K;
    v.smem_bytes = kSmem;
    return v;
  }
};


// ---------------------------------------------------------------------------
// One step of a 3D single-stage program on rows of four-point vectors
// ---------------------------------------------------------------------------
// For programs whose stencil is a star of reach 1 (every load moves along at
// most one axis, by at most one point) and whose step rolls the state by one
// point (heat-like programs), in FP32 or FP16 storage.  A warp covers 128
// consecutive points of a row.  A lane owns the four rolled destinations
// x0..x0+3 (x0 a multiple of four) and stores them with one vector store;
// their sources are x0-1..x0+2, whose x-neighbours are x0-2..x0+3: one
// aligned vector load of x0..x0+3 and the last two values of the lane on the
// left (warp shuffles; lane 0 loads those two itself).  The rows y-1 and y+1
// and the planes z-1 and z+1 arrive the same way, so a thread issues about
// one vector load per point it updates instead of seven scalar loads, and
// every value the stage functor reads comes from registers.  Results are
// those of the generic stage kernel, bit for bit.

// four consecutive storage elements: one aligned vector load or store
template <class S> struct Quad;
template <> struct Quad<float> {
  static __device__ __forceinline__ void get(const float* p, float, float v[4]) {
    const float4 q = __ldg(reinterpret_cast<const float4*>(p));
    v[0] = q.x;
    v[1] = q.y;
    v[2] = q.z;
    v[3] = q.w;
  }
  static __device__ __forceinline__ void put(float* p, const float v[4], float) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  }
};
template <> struct Quad<__half> {
  static __device__ __forceinline__ void get(const __half* p, float scale, float v[4]) {
    const uint2 q = __ldg(reinterpret_cast<const uint2*>(p));
    __half h[4];
    memcpy(h, &q, sizeof q);
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = Storage<__half, float>::load(h[i], scale);
  }
  static __device__ __forceinline__ void put(__half* p, const float v[4], float inv_scale) {
    __half h[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) h[i] = Storage<__half, float>::store(v[i], inv_scale);
    uint2 q;
    memcpy(&q, h, sizeof q);
    *reinterpret_cast<uint2*>(p) = q;
  }
};

// Accessor of one point (row R of the thread, element E of its four): the
// centre plane's rows y-1 .. y+RY hold x0-2 .. x0+3, the planes z-1 and z+1
// the thread's own rows.  Every index is a compile-time constant.
template <class T, int NF, int RY, int R, int E>
struct QuadAccess {
  const T (&c)[NF][RY + 2][6];
  const T (&z)[NF][2][RY][4];
  T (&out)[NF][RY][4];
  template <int F, int D0, int D1, int D2>
  __device__ __forceinline__ T ld() const {
    static_assert((D0 != 0) + (D1 != 0) + (D2 != 0) <= 1, "star stencils only");
    static_assert(D0 >= -1 && D0 <= 1 && D1 >= -1 && D1 <= 1 && D2 >= -1 && D2 <= 1, "reach 1 only");
    if constexpr (D0 == 0)
      return c[F][R + 1 + D1][E + 1 + D2];
    else
      return z[F][D0 > 0 ? 1 : 0][R][E];
  }
  template <int F>
  __device__ __forceinline__ void st(T v) const {
    out[F][R][E] = v;
  }
};

template <int... I, class Fn>
__device__ __forceinline__ void static_for(std::integer_sequence<int, I...>, Fn&& fn) {
  (fn(std::integral_constant<int, I>{}), ...);
}

template <class M, class S, class Stage, int NF, int RY, int BW>
__global__ void __launch_bounds__(32 * BW) quad3d_kernel(const __grid_constant__ FgbLaunch L) {
  using T = typename M::T;
  constexpr unsigned kFull = 0xffffffffu;
  const int n0 = L.n[0], n1 = L.n[1], n2 = L.n[2];
  const int lane = threadIdx.x;
  const int x0 = (blockIdx.x * 32 + lane) * 4;
  const bool active = x0 < n2;
  const int y0 = (blockIdx.y * BW + threadIdx.y) * RY;   // first source row (warp-uniform)
  const int p0 = blockIdx.z;                             // source plane
  const int xl4 = x0 >= 4 ? x0 - 4 : x0 - 4 + n2;        // lane 0's left vector x0-4 .. x0-1
  auto row_at = [&](int p, int y) -> uint32_t { return ((uint32_t)p * (uint32_t)n1 + (uint32_t)y) * (uint32_t)n2; };
  // window x0-2 .. x0+3 of one row (all lanes take part in the shuffles;
  // lane 0 loads the vector to its left)
  auto window = [&](const S* a, float scale, uint32_t row, T w[6]) {
    T v[4] = {T(0), T(0), T(0), T(0)};
    if (active) Quad<S>::get(a + row + x0, scale, v);
    T l2 = __shfl_up_sync(kFull, v[2], 1);
    T l3 = __shfl_up_sync(kFull, v[3], 1);
    if (lane == 0 && active) {
      T u[4];
      Quad<S>::get(a + row + xl4, scale, u);
      l2 = u[2];
      l3 = u[3];
    }
    w[0] = l2;
    w[1] = l3;
#pragma unroll
    for (int i = 0; i < 4; ++i) w[2 + i] = v[i];
  };
  const int pm = p0 > 0 ? p0 - 1 : n0 - 1, pp = p0 + 1 < n0 ? p0 + 1 : 0;
  // rows y0-1 .. y0+RY, wrapped: one division, then steps
  int yr[RY + 2];
  yr[0] = pmod(y0 - 1, n1);
#pragma unroll
  for (int r = 1; r < RY + 2; ++r) yr[r] = yr[r - 1] + 1 == n1 ? 0 : yr[r - 1] + 1;
  T c[NF][RY + 2][6];
  T z[NF][2][RY][4];
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    const S* a = static_cast<const S*>(L.in[f]);
    const float sc = L.scale[f];
#pragma unroll
    for (int r = 0; r < RY + 2; ++r) window(a, sc, row_at(p0, yr[r]), c[f][r]);
#pragma unroll
    for (int r = 0; r < RY; ++r) {
#pragma unroll
      for (int d = 0; d < 2; ++d) {
        T w[6];
        window(a, sc, row_at(d ? pp : pm, yr[r + 1]), w);   // x0-2 .. x0+3; the sources are x0-1 .. x0+2
#pragma unroll
        for (int i = 0; i < 4; ++i) z[f][d][r][i] = w[1 + i];
      }
    }
  }
  T out[NF][RY][4];
  const typename M::U* U = static_cast<const typename M::U*>(L.uniforms);
  static_for(std::make_integer_sequence<int, RY>{}, [&](auto rc) {
    constexpr int R = decltype(rc)::value;
    static_for(std::make_integer_sequence<int, 4>{}, [&](auto ec) {
      constexpr int E = decltype(ec)::value;
      QuadAccess<T, NF, RY, R, E> acc{c, z, out};
      eval<M, Stage>(acc, U);
    });
  });
  if (!active) return;
#pragma unroll
  for (int r = 0; r < RY; ++r) {
    if (y0 + r >= n1) break;
    const int yd = y0 + r + 1 < n1 ? y0 + r + 1 : 0;    // rolled by one point (y0 + r < n1)
#pragma unroll
    for (int f = 0; f < NF; ++f)
      Quad<S>::put(static_cast<S*>(L.out[f]) + row_at(pp, yd) + x0, out[f][r], L.inv_scale[f]);
  }
}

template <class Prog, int P, class Stage, int RY, int BW>
struct Quad3dVariant {
  using M = typename Precision<P>::M;
  using S = typename Precision<P>::S;
  static cudaError_t launch(const FgbLaunch* L, cudaStream_t stream) {
    const dim3 grid((L->n[2] + 127) / 128, (L->n[1] + BW * RY - 1) / (BW * RY), L->n[0]);
    quad3d_kernel<M, S, Stage, Prog::kFields, RY, BW><<<grid, dim3(32, BW), 0, stream>>>(*L);
    return cudaGetLastError();
  }
  static FgbFusedVariant describe() {
    FgbFusedVariant v;
    v.x_multiple = 4;
    v.launch = &launch;
    v.tile_x = 128;
    v.tile_y = BW * RY;
    v.steps = 1;
    v.smem_bytes = 0;
    return v;
  }
};


// ---------------------------------------------------------------------------
// One step of a 3D single-stage program, marching along z through shared memory
// ---------------------------------------------------------------------------
// The same programs and the same four-point row vectors as quad3d_kernel,
// but a CTA walks a chunk of planes and every plane of its tile (with one
// row above and below and four points to the left) arrives once, by
// cp.async into a ring of shared-memory slots, P planes ahead of the plane
// being updated.  A thread then reads its centre window (x0-2 .. x0+3 of
// rows y-1 .. y+RY) and its rows of the planes z-1 and z+1 from shared
// memory.  L2 serves each value about (rows + 2) / rows times instead of
// the one-plane kernel's three and a quarter, and the copies in flight do
// not hold registers.  Results are the generic stage kernel's.
template <class S>
__device__ __forceinline__ void cp_async4(S* dst, const S* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  if constexpr (sizeof(S) == 4)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// four consecutive storage elements from shared memory (aligned)
template <class S> struct QuadSm;
template <> struct QuadSm<float> {
  static __device__ __forceinline__ void get(const float* p, float, float v[4]) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    v[0] = q.x;
    v[1] = q.y;
    v[2] = q.z;
    v[3] = q.w;
  }
};
template <> struct QuadSm<__half> {
  static __device__ __forceinline__ void get(const __half* p, float scale, float v[4]) {
    const uint2 q = *reinterpret_cast<const uint2*>(p);
    __half h[4];
    memcpy(h, &q, sizeof q);
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = Storage<__half, float>::load(h[i], scale);
  }
};

template <class S, int NF, int RY, int BW, int P>
struct ZringLayout {
  static constexpr int kRows = BW * RY + 2;        // the tile's rows and one row either side
  static constexpr int kRow = 132;                 // x_lo-4 .. x_lo+127
  static constexpr int kSlots = P + 3;             // planes z-1, z, z+1 and P ahead
  static constexpr int kPlane = NF * kRows * kRow; // elements of one slot
  static constexpr size_t kBytes = (size_t)kSlots * kPlane * sizeof(S);
};

template <class M, class S, class Stage, int NF, int RY, int BW, int P>
__global__ void __launch_bounds__(32 * BW) zring3d_kernel(const __grid_constant__ FgbLaunch L) {
  using T = typename M::T;
  using Lay = ZringLayout<S, NF, RY, BW, P>;
  constexpr int NS = Lay::kSlots, ROWS = Lay::kRows, RW = Lay::kRow;
  extern __shared__ __align__(16) unsigned char zr_smem[];
  S* sm = reinterpret_cast<S*>(zr_smem);
  const int n0 = L.n[0], n1 = L.n[1], n2 = L.n[2];
  const int lane = threadIdx.x, w = threadIdx.y, tid = w * 32 + lane;
  const int xlo = blockIdx.x * 128, ylo = blockIdx.y * (BW * RY);
  const int chunk = (n0 + gridDim.z - 1) / gridDim.z;
  const int za = blockIdx.z * chunk, zb = za + chunk < n0 ? za + chunk : n0;
  if (za >= zb) return;
  // four-point pieces of one plane: per row, the left halo piece
  // (x_lo-4 .. x_lo-1, wrapped) and the 32 pieces of x_lo .. x_lo+127.  A
  // thread copies the same pieces of every plane and field: their offsets
  // within a plane (global and in its slot) are formed once.
  constexpr int kPieces = ROWS * 33, kMine = (kPieces + 32 * BW - 1) / (32 * BW);
  uint32_t src_off[kMine];
  int dst_off[kMine];
#pragma unroll
  for (int j = 0; j < kMine; ++j) {
    const int i = tid + j * 32 * BW;
    const int r = i / 33, k = i - r * 33;
    const int x = k == 0 ? (xlo == 0 ? n2 - 4 : xlo - 4) : xlo + 4 * (k - 1);
    // pieces past the rows or right of the grid are not copied (the
    // columns right of the grid are read by idle lanes only)
    dst_off[j] = i < kPieces && x < n2 ? r * RW + 4 * k : -1;
    src_off[j] = (uint32_t)pmod(ylo - 1 + r, n1) * (uint32_t)n2 + (uint32_t)x;
  }
  const uint32_t plane_elems = (uint32_t)n1 * (uint32_t)n2;
  auto issue = [&](int q) {   // plane q (unwrapped, za-1 <= q) into its slot
    const int slot = (q - za + 1) % NS;
    const uint32_t base = (uint32_t)pmod(q, n0) * plane_elems;   // P may exceed the grid's depth
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      const S* a = static_cast<const S*>(L.in[f]) + base;
      S* d = sm + (size_t)slot * Lay::kPlane + f * ROWS * RW;
#pragma unroll
      for (int j = 0; j < kMine; ++j)
        if (dst_off[j] >= 0) cp_async4(d + dst_off[j], a + src_off[j]);
    }
    cp_async_commit();
  };
  // prologue: planes za-1, za, then za+1 .. za+P, one group each
  issue(za - 1);
  issue(za);
#pragma unroll 1
  for (int q = za + 1; q <= za + P; ++q) issue(q);
  const int x0 = xlo + 4 * lane;
  const bool active = x0 < n2;
  const int yt = ylo + w * RY;   // the thread's first row (source)
  const typename M::U* U = static_cast<const typename M::U*>(L.uniforms);
#pragma unroll 1
  for (int p = za; p < zb; ++p) {
    cp_async_wait<P - 1>();   // planes up to p+1 have landed (this thread's pieces)
    __syncthreads();          // ... everyone's, and plane p-2's slot is free
    issue(p + 1 + P);         // (beyond the chunk the copies are unused but harmless)
    const S* cz = sm + (size_t)((p - za + 1) % NS) * Lay::kPlane;
    const S* zm = sm + (size_t)((p - za) % NS) * Lay::kPlane;
    const S* zp = sm + (size_t)((p - za + 2) % NS) * Lay::kPlane;
    // each row: the thread's vector x0 .. x0+3, and the values to its left
    // from the lane on the left (lane 0: from the row's halo)
    T c[NF][RY + 2][6];
    T z[NF][2][RY][4];
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      const float sc = L.scale[f];
#pragma unroll
      for (int r = 0; r < RY + 2; ++r) {
        const S* row = cz + (f * ROWS + w * RY + r) * RW;
        T v[4];
        QuadSm<S>::get(row + 4 + 4 * lane, sc, v);
        T l2 = __shfl_up_sync(0xffffffffu, v[2], 1), l3 = __shfl_up_sync(0xffffffffu, v[3], 1);
        if (lane == 0) {
          l2 = Storage<S, T>::load(row[2], sc);
          l3 = Storage<S, T>::load(row[3], sc);
        }
        c[f][r][0] = l2;
        c[f][r][1] = l3;
#pragma unroll
        for (int i = 0; i < 4; ++i) c[f][r][2 + i] = v[i];
      }
#pragma unroll
      for (int r = 0; r < RY; ++r) {
#pragma unroll
        for (int d = 0; d < 2; ++d) {
          const S* row = (d ? zp : zm) + (f * ROWS + w * RY + 1 + r) * RW;
          T v[4];
          QuadSm<S>::get(row + 4 + 4 * lane, sc, v);
          T l3 = __shfl_up_sync(0xffffffffu, v[3], 1);
          if (lane == 0) l3 = Storage<S, T>::load(row[3], sc);
          z[f][d][r][0] = l3;
#pragma unroll
          for (int i = 0; i < 3; ++i) z[f][d][r][1 + i] = v[i];
        }
      }
    }
    T out[NF][RY][4];
    static_for(std::make_integer_sequence<int, RY>{}, [&](auto rc) {
      constexpr int R = decltype(rc)::value;
      static_for(std::make_integer_sequence<int, 4>{}, [&](auto ec) {
        constexpr int E = decltype(ec)::value;
        QuadAccess<T, NF, RY, R, E> acc{c, z, out};
        eval<M, Stage>(acc, U);
      });
    });
    if (active) {
      const int pd = p + 1 < n0 ? p + 1 : 0;   // rolled by one point
#pragma unroll
      for (int r = 0; r < RY; ++r) {
        if (yt + r >= n1) break;
        const int yd = yt + r + 1 < n1 ? yt + r + 1 : 0;
#pragma unroll
        for (int f = 0; f < NF; ++f)
          Quad<S>::put(static_cast<S*>(L.out[f]) + ((uint32_t)pd * (uint32_t)n1 + (uint32_t)yd) * (uint32_t)n2 + x0,
                       out[f][r], L.inv_scale[f]);
      }
    }
  }
  cp_async_wait<0>();   // no copy may land after the block's shared memory is released
}

template <class Prog, int P, class Stage, int RY, int BW, int PF>
struct Zring3dVariant {
  using M = typename Precision<P>::M;
  using S = typename Precision<P>::S;
  using Lay = ZringLayout<S, Prog::kFields, RY, BW, PF>;
  static cudaError_t launch(const FgbLaunch* L, cudaStream_t stream) {
    auto kern = zring3d_kernel<M, S, Stage, Prog::kFields, RY, BW, PF>;
    static int resident = 0;   // CTAs of this kernel the device holds at once
    if (resident == 0) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Lay::kBytes);
      int dev = 0, sms = 0, per_sm = 0;
      if (e == cudaSuccess) e = cudaGetDevice(&dev);
      if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * BW, Lay::kBytes);
      if (e != cudaSuccess) return e;
      resident = sms * per_sm > 0 ? sms * per_sm : 1;
    }
    const int gx = (L->n[2] + 127) / 128, gy = (L->n[1] + BW * RY - 1) / (BW * RY);
    // at most one wave of CTAs, each walking a chunk of at least 8 planes
    const int want = resident / (gx * gy) > 1 ? resident / (gx * gy) : 1;
    const int most = L->n[0] / 8 > 1 ? L->n[0] / 8 : 1;
    const int gz = want < most ? want : most;
    kern<<<dim3(gx, gy, gz), dim3(32, BW), Lay::kBytes, stream>>>(*L);
    return cudaGetLastError();
  }
  static FgbFusedVariant describe() {
    FgbFusedVariant v;
    v.x_multiple = 4;
    v.launch = &launch;
    v.tile_x = 128;
    v.tile_y = BW * RY;
    v.steps = 1;
    v.smem_bytes = Lay::kBytes;
    return v;
  }
};

}  // namespace fgb

#include "fgb_fused_ms.cuh"
