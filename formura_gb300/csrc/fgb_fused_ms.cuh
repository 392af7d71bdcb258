// One step of a multi-stage 3D program in one launch (2.5D streaming).
//
// A multi-stage step (HLLC Euler: face states and their divergence, Riemann
// fluxes, update) normally runs one kernel per stage and passes each stage's
// arrays to the next through HBM: for the Euler step in FP32 that is about
// 430 bytes of DRAM traffic per point against 40 bytes of state.  Here one
// CTA owns a TY x TX column of the grid and streams along the slowest axis.
// Every stage's arrays live in shared memory, in a ring of the planes that
// later stages still read; the state arrives plane by plane into a ring of
// its own.  In each iteration the CTA loads one state plane, then runs the
// stages in order, each on the newest plane it can complete, over the part
// of the column (with its halo) that later stages read.  Only the state is
// read from and written to HBM.
//
// The halo and ring depths follow from where each stage reads the arrays of
// the earlier stages and the state (the generator's StageReads table).  The
// stage functors are the generated ones, unchanged: they see an accessor
// that maps array and state loads to the shared-memory rings.  Every tile
// shape gives the same bits; against the stage-per-kernel path the FP32
// results agree to rounding, since nvcc contracts products and sums into
// FMAs differently in the two kernels.
#pragma once

namespace fgb {

template <class Prog>
struct MsGeometry {
  using R = typename Prog::Reads;
  static constexpr int NS = Prog::kStages;
  struct Ext {
    int lo[NS][3], hi[NS][3];  // points a stage computes, relative to the output tile
    int slo[3], shi[3];        // state points the stages read
  };
  static constexpr bool reads(int c, int s) { return R::kReadLo[c][s][0] <= R::kReadHi[c][s][0]; }
  static constexpr bool reads_state(int s) { return R::kStateLo[s][0] <= R::kStateHi[s][0]; }
  static constexpr Ext compute() {
    Ext e{};
    for (int a = 0; a < 3; ++a) e.lo[NS - 1][a] = e.hi[NS - 1][a] = 0;
    for (int s = NS - 2; s >= 0; --s) {
      for (int a = 0; a < 3; ++a) {
        int lo = 1 << 20, hi = -(1 << 20);
        for (int c = s + 1; c < NS; ++c) {
          if (!reads(c, s)) continue;
          lo = e.lo[c][a] + R::kReadLo[c][s][a] < lo ? e.lo[c][a] + R::kReadLo[c][s][a] : lo;
          hi = e.hi[c][a] + R::kReadHi[c][s][a] > hi ? e.hi[c][a] + R::kReadHi[c][s][a] : hi;
        }
        e.lo[s][a] = lo;
        e.hi[s][a] = hi;
      }
    }
    for (int a = 0; a < 3; ++a) {
      int lo = 1 << 20, hi = -(1 << 20);
      for (int s = 0; s < NS; ++s) {
        if (!reads_state(s)) continue;
        lo = e.lo[s][a] + R::kStateLo[s][a] < lo ? e.lo[s][a] + R::kStateLo[s][a] : lo;
        hi = e.hi[s][a] + R::kStateHi[s][a] > hi ? e.hi[s][a] + R::kStateHi[s][a] : hi;
      }
      e.slo[a] = lo;
      e.shi[a] = hi;
    }
    return e;
  }
  static constexpr Ext E = compute();
  // planes of stage s's arrays held at once: from its newest plane back to
  // the oldest plane a later stage still reads in the same iteration
  static constexpr int ring(int s) {
    int oldest = E.hi[s][0];
    for (int c = s + 1; c < NS; ++c)
      if (reads(c, s) && E.hi[c][0] + R::kReadLo[c][s][0] < oldest) oldest = E.hi[c][0] + R::kReadLo[c][s][0];
    return E.hi[s][0] - oldest + 1;
  }
  static constexpr int state_oldest() {
    int oldest = E.shi[0];
    for (int s = 0; s < NS; ++s)
      if (reads_state(s) && E.hi[s][0] + R::kStateLo[s][0] < oldest) oldest = E.hi[s][0] + R::kStateLo[s][0];
    return oldest;
  }
  static constexpr int kStateRing = E.shi[0] - state_oldest() + 1;
  // iterations before the first output plane (stage s first computes the
  // plane E.lo[s][0] below it)
  static constexpr int lead() {
    int m = 0;
    for (int s = 0; s < NS; ++s) m = E.hi[s][0] - E.lo[s][0] > m ? E.hi[s][0] - E.lo[s][0] : m;
    return m;
  }
  static constexpr int kLead = lead();
};

// shared-memory layout for a TY x TX output tile: the state ring, then for
// every array its stage's ring
template <class Prog, class T, int TY, int TX>
struct MsLayout {
  using G = MsGeometry<Prog>;
  static constexpr int NS = Prog::kStages;
  static constexpr int SY = TY + G::E.shi[1] - G::E.slo[1];
  static constexpr int SX = TX + G::E.shi[2] - G::E.slo[2];
  static constexpr int sy(int s) { return TY + G::E.hi[s][1] - G::E.lo[s][1]; }
  static constexpr int sx(int s) { return TX + G::E.hi[s][2] - G::E.lo[s][2]; }
  static constexpr size_t kStateElems = (size_t)Prog::kFields * G::kStateRing * SY * SX;
  static constexpr size_t mid_elems(int k) {
    const int s = Prog::Reads::kMidStage[k];
    return (size_t)G::ring(s) * sy(s) * sx(s);
  }
  static constexpr size_t mid_offset(int k) {
    size_t o = kStateElems;
    for (int i = 0; i < k; ++i) o += mid_elems(i);
    return o;
  }
  static constexpr size_t kElems = mid_offset(Prog::kMids);
  static constexpr size_t kBytes = kElems * sizeof(T);
};

template <int Q>
__device__ __forceinline__ int ring_slot(int plane) {
  return (plane + 64 * Q) % Q;   // planes start at most a few below zero
}

// Accessor of one point (tile-relative row ly, column lx, global plane q):
// state and array loads come from the shared-memory rings, array stores go
// to the ring of the point's stage, state stores to HBM rolled by the
// program's shift (Templates.hs:346).
template <class Prog, class S, class T, int TY, int TX>
struct MsAccess {
  using G = MsGeometry<Prog>;
  using Lay = MsLayout<Prog, T, TY, TX>;
  T* sm;
  const FgbLaunch& L;
  int q, ly, lx;   // plane (global, unwrapped), row and column relative to the tile
  int y0, x0;      // the tile's origin in the grid
  template <int F, int D0, int D1, int D2>
  __device__ __forceinline__ T ld() const {
    constexpr int Q = G::kStateRing, lo1 = G::E.slo[1], lo2 = G::E.slo[2];
    const int slot = ring_slot<Q>(q + D0);
    return sm[((F * Q + slot) * Lay::SY + (ly + D1 - lo1)) * Lay::SX + (lx + D2 - lo2)];
  }
  template <int K, int D0, int D1, int D2>
  __device__ __forceinline__ T ldm() const {
    constexpr int s = Prog::Reads::kMidStage[K];
    constexpr int Q = G::ring(s), lo1 = G::E.lo[s][1], lo2 = G::E.lo[s][2], SY = Lay::sy(s), SX = Lay::sx(s);
    constexpr size_t off = Lay::mid_offset(K);
    const int slot = ring_slot<Q>(q + D0);
    return sm[off + ((size_t)slot * SY + (ly + D1 - lo1)) * SX + (lx + D2 - lo2)];
  }
  template <int K>
  __device__ __forceinline__ void stm(T v) const {
    constexpr int s = Prog::Reads::kMidStage[K];
    constexpr int Q = G::ring(s), lo1 = G::E.lo[s][1], lo2 = G::E.lo[s][2], SY = Lay::sy(s), SX = Lay::sx(s);
    constexpr size_t off = Lay::mid_offset(K);
    sm[off + ((size_t)ring_slot<Q>(q) * SY + (ly - lo1)) * SX + (lx - lo2)] = v;
  }
  template <int F>
  __device__ __forceinline__ void st(T v) const {
    const int n0 = L.n[0], n1 = L.n[1], n2 = L.n[2];
    const int i0 = pmod(q + Prog::kShift, n0), i1 = pmod(y0 + ly + Prog::kShift, n1);
    const int i2 = pmod(x0 + lx + Prog::kShift, n2);
    static_cast<S*>(L.out[F])[((uint32_t)i0 * (uint32_t)n1 + (uint32_t)i1) * (uint32_t)n2 + (uint32_t)i2] =
        Storage<S, T>::store(v, L.inv_scale[F]);
  }
};

// Stage s on its plane of iteration p, over its part of the column.
template <class M, class Prog, class S, int TY, int TX, int s, class Stage>
__device__ __forceinline__ void ms_stage(typename M::T* sm, const FgbLaunch& L, int p, int za, int zb, int y0,
                                         int x0, const typename M::U* __restrict__ U) {
  using G = MsGeometry<Prog>;
  using Lay = MsLayout<Prog, typename M::T, TY, TX>;
  constexpr int hi0 = G::E.hi[s][0], lo0 = G::E.lo[s][0], lo1 = G::E.lo[s][1], lo2 = G::E.lo[s][2];
  const int q = p + hi0;
  if (q < za + lo0) return;
  constexpr int W = Lay::sx(s), N = Lay::sy(s) * Lay::sx(s);
  const int nthreads = blockDim.x * blockDim.y;
  for (int i = threadIdx.y * blockDim.x + threadIdx.x; i < N; i += nthreads) {
    const int ly = lo1 + i / W, lx = lo2 + i % W;
    if constexpr (s == Prog::kStages - 1) {
      // the last stage writes the state: only the tile's points inside the grid
      if (y0 + ly >= L.n[1] || x0 + lx >= L.n[2]) continue;
    }
    MsAccess<Prog, S, typename M::T, TY, TX> a{sm, L, q, ly, lx, y0, x0};
    eval<M, Stage>(a, U);
  }
}

// One state plane (global plane q, wrapped) into its ring slot, as compute values.
template <class Prog, class S, class T, int TY, int TX>
__device__ __forceinline__ void ms_load_plane(T* sm, const FgbLaunch& L, int q, int y0, int x0) {
  using G = MsGeometry<Prog>;
  using Lay = MsLayout<Prog, T, TY, TX>;
  constexpr int Q = G::kStateRing, lo1 = G::E.slo[1], lo2 = G::E.slo[2];
  const int n0 = L.n[0], n1 = L.n[1], n2 = L.n[2];
  const int i0 = pmod(q, n0);
  const int slot = ring_slot<Q>(q);
  const int nthreads = blockDim.x * blockDim.y;
  constexpr int N = Lay::SY * Lay::SX;
  for (int i = threadIdx.y * blockDim.x + threadIdx.x; i < N; i += nthreads) {
    const int ry = i / Lay::SX, rx = i % Lay::SX;
    const int gy = pmod(y0 + lo1 + ry, n1), gx = pmod(x0 + lo2 + rx, n2);
    const uint32_t k = ((uint32_t)i0 * (uint32_t)n1 + (uint32_t)gy) * (uint32_t)n2 + (uint32_t)gx;
#pragma unroll
    for (int f = 0; f < Prog::kFields; ++f)
      sm[((f * Q + slot) * Lay::SY + ry) * Lay::SX + rx] =
          Storage<S, T>::load(ro_load(static_cast<const S*>(L.in[f]) + k), L.scale[f]);
  }
}

template <class M, class Prog, class S, int TY, int TX, class... Stages>
__global__ void __launch_bounds__(256) ms3d_kernel(const __grid_constant__ FgbLaunch L) {
  using T = typename M::T;
  using G = MsGeometry<Prog>;
  extern __shared__ __align__(16) unsigned char ms_smem[];
  T* sm = reinterpret_cast<T*>(ms_smem);
  const int y0 = blockIdx.y * TY, x0 = blockIdx.x * TX;
  const int n0 = L.n[0];
  const int chunk = (n0 + gridDim.z - 1) / gridDim.z;
  const int za = blockIdx.z * chunk, zb = za + chunk < n0 ? za + chunk : n0;
  if (za >= zb) return;
  const typename M::U* U = static_cast<const typename M::U*>(L.uniforms);
  constexpr int lead = G::kLead, oldest = G::state_oldest(), newest = G::E.shi[0];
  const int pfirst = za - lead;
  // the state planes the first iteration reads besides the one it loads
  for (int q = pfirst + oldest; q < pfirst + newest; ++q) ms_load_plane<Prog, S, T, TY, TX>(sm, L, q, y0, x0);
  for (int p = pfirst; p < zb; ++p) {
    __syncthreads();   // the slot about to be loaded is no longer read
    ms_load_plane<Prog, S, T, TY, TX>(sm, L, p + newest, y0, x0);
    __syncthreads();
    ((ms_stage<M, Prog, S, TY, TX, Stages::kIndex, Stages>(sm, L, p, za, zb, y0, x0, U), __syncthreads()), ...);
  }
}

template <class Prog, int P, int TY, int TX, class... Stages>
struct Ms3dVariant {
  static_assert(((Stages::kIndex == Prog::kStages - 1 || !Stages::kWritesState) && ...),
                "only the last stage writes the state");
  using M = typename Precision<P>::M;
  using S = typename Precision<P>::S;
  using Lay = MsLayout<Prog, typename M::T, TY, TX>;
  static constexpr size_t kSmem = Lay::kBytes;
  static cudaError_t launch(const FgbLaunch* L, cudaStream_t stream) {
    auto kern = ms3d_kernel<M, Prog, S, TY, TX, Stages...>;
    static bool configured = false;
    if (!configured) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
      if (e != cudaSuccess) return e;
      configured = true;
    }
    const int gx = (L->n[2] + TX - 1) / TX, gy = (L->n[1] + TY - 1) / TY;
    // about eight CTAs per SM in all, and chunks at least 8 * lead planes deep
    const int want = (8 * 152 + gx * gy - 1) / (gx * gy);
    const int lead = MsGeometry<Prog>::kLead > 0 ? MsGeometry<Prog>::kLead : 1;
    const int most = L->n[0] / (8 * lead) > 1 ? L->n[0] / (8 * lead) : 1;
    const int gz = want < most ? want : most;
    kern<<<dim3(gx, gy, gz), dim3(32, 8), kSmem, stream>>>(*L);
    return cudaGetLastError();
  }
  static FgbFusedVariant describe() {
    FgbFusedVariant v;
    v.x_multiple = 1;
    v.launch = &launch;
    v.tile_x = TX;
    v.tile_y = TY;
    v.steps = 1;
    v.smem_bytes = kSmem;
    return v;
  }
};

}  // namespace fgb
