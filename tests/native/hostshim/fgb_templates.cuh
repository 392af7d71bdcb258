// Host stand-in for the kernel templates, used by the CPU tests: it compiles
// a generated program file (formura_gb300/_gen/prog_<name>.cu) with g++ and
// runs its stage functors, and the functors of its adjoint, over a small
// periodic grid one point at a time.  The arithmetic policy rounds every
// operation once in IEEE binary64 (compile with -ffp-contract=off), which is
// what the exact FP64 policy of the device computes.  Entry points, per
// program NAME defined in the file:
//   host_forward_NAME(n, U, u, out)            one step: u -> out (rolled by shift)
//   host_backward_NAME(n, U, u, lnext, lprev)  one adjoint step at u (0), or 1
//                                              when the program has no adjoint
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#define __device__
#define __host__
#define __forceinline__ inline

namespace fgb {
template <class Rec, class... Pairs>
struct AdjointStages {};
template <class Partial, class Gather>
struct AdjointStagePair {
  using P1 = Partial;
  using P2 = Gather;
};
template <class... Parts>
struct AdjParts {};
// the program's own forward stages, when the forward step stores other arrays
template <class... S>
struct StageTypes {};
}  // namespace fgb

namespace hostshim {

struct Exact {
  using T = double;
  using U = double;
  using Deriv = Exact;   // derivative terms: also one rounding per operation here
  static T add(T a, T b) { return a + b; }
  static T sub(T a, T b) { return a - b; }
  static T mul(T a, T b) { return a * b; }
  static T div(T a, T b) { return a / b; }
  // the reference's separately rounded operations, which the device's
  // shortened forms (or their IEEE fallback) reproduce
  static T fma(T a, T b, T c, bool&) { return a * b + c; }
  static T divu(T x, T c, T, bool&) { return x / c; }
  static T rcp(T b) { return 1.0 / b; }
  static bool lt(T a, T b) { return a < b; }
  static bool gt(T a, T b) { return a > b; }
  static bool le(T a, T b) { return a <= b; }
  static bool ge(T a, T b) { return a >= b; }
  static bool eq(T a, T b) { return a == b; }
  static bool ne(T a, T b) { return a != b; }
  static T divr(T a, T b, T, bool&) { return a / b; }
  static T neg(T a) { return -a; }
  static T one_minus(T x) { return 1.0 - x; }
  static T sqrt(T a) { return std::sqrt(a); }
  static T fabs(T a) { return std::fabs(a); }
  static T exp(T a) { return std::exp(a); }
  static T log(T a) { return std::log(a); }
  static T sin(T a) { return std::sin(a); }
  static T cos(T a) { return std::cos(a); }
  static T pow(T a, T b) { return std::pow(a, b); }
};

struct Grid {
  int n[3];
  size_t cells;
  const double* U;
  const double* u;
  double* out;
  std::vector<double> mids, lmids, pairs;
  const double* lnext;
  double* lprev;
  static int wrap(int i, int m) { return ((i % m) + m) % m; }
  size_t lin(int i0, int i1, int i2) const {
    return ((size_t)wrap(i0, n[0]) * n[1] + wrap(i1, n[1])) * n[2] + wrap(i2, n[2]);
  }
};

template <int DIM, int SHIFT>
struct Fwd {
  Grid* g;
  int p0, p1, p2;
  template <int F, int D0, int D1, int D2>
  double ld() const { return g->u[F * g->cells + g->lin(p0 + D0, p1 + D1, p2 + D2)]; }
  template <int K, int D0, int D1, int D2>
  double ldm() const { return g->mids[K * g->cells + g->lin(p0 + D0, p1 + D1, p2 + D2)]; }
  template <int F>
  void st(double v) const {
    g->out[F * g->cells + g->lin(p0 + (DIM >= 3 ? SHIFT : 0), p1 + (DIM >= 2 ? SHIFT : 0), p2 + SHIFT)] = v;
  }
  template <int K>
  void stm(double v) const { g->mids[K * g->cells + g->lin(p0, p1, p2)] = v; }
};

// single-stage adjoint (one pass)
struct Adj1 {
  Grid* g;
  int p0, p1, p2;
  template <int F, int D0, int D1, int D2>
  double ld() const { return g->u[F * g->cells + g->lin(p0 + D0, p1 + D1, p2 + D2)]; }
  template <int F, int D0, int D1, int D2>
  double ldl() const { return g->lnext[F * g->cells + g->lin(p0 + D0, p1 + D1, p2 + D2)]; }
  template <int F>
  void stl(double v) const { g->lprev[F * g->cells + g->lin(p0, p1, p2)] = v; }
};

struct Partial {
  Grid* g;
  int p0, p1, p2;
  template <int F, int D0, int D1, int D2>
  double ld() const { return g->u[F * g->cells + g->lin(p0 + D0, p1 + D1, p2 + D2)]; }
  template <int K, int D0, int D1, int D2>
  double ldm() const { return g->mids[K * g->cells + g->lin(p0 + D0, p1 + D1, p2 + D2)]; }
  template <int F>
  void st(double) const {}
  template <int K>
  void stm(double) const {}
  template <int F, int D0, int D1, int D2>
  double ldl() const { return g->lnext[F * g->cells + g->lin(p0 + D0, p1 + D1, p2 + D2)]; }
  template <int K>
  double ldlm() const { return g->lmids[K * g->cells + g->lin(p0, p1, p2)]; }
  template <int J>
  void stp(double v) const { g->pairs[J * g->cells + g->lin(p0, p1, p2)] = v; }
};

struct Gather {
  Grid* g;
  int p0, p1, p2;
  template <int J, int D0, int D1, int D2>
  double ldp() const { return g->pairs[J * g->cells + g->lin(p0 + D0, p1 + D1, p2 + D2)]; }
  template <int G, bool FIRST>
  void accs(double v) const {
    double& a = g->lprev[G * g->cells + g->lin(p0, p1, p2)];
    a = FIRST ? v : v + a;
  }
  template <int K, bool FIRST>
  void accm(double v) const {
    double& a = g->lmids[K * g->cells + g->lin(p0, p1, p2)];
    a = FIRST ? v : v + a;
  }
};

// sum J of a partial-sum functor at its point; the others are dropped
template <int J>
struct Capture : Partial {
  double* out;
  template <int J2>
  void stp(double v) const {
    if (J2 == J) *out = v;
  }
};

// gather of a linear stage: the partial sums are formed where they are read
template <class Parts>
struct Direct;
template <class... Parts>
struct Direct<fgb::AdjParts<Parts...>> : Gather {
  template <int J, int D0, int D1, int D2>
  double ldp() const {
    double v = 0.0;
    const Capture<J> c{{g, p0 + D0, p1 + D1, p2 + D2}, &v};
    (Parts::template run<Exact>(c, g->U), ...);
    return v;
  }
};

template <class Acc, class F>
void sweep(Grid& g) {
  for (int i = 0; i < g.n[0]; ++i)
    for (int j = 0; j < g.n[1]; ++j)
      for (int k = 0; k < g.n[2]; ++k) {
        Acc a{&g, i, j, k};
        F::template run<Exact>(a, g.U);
      }
}

// The forward stages the adjoint recomputes its arrays with, and how many
// arrays they store: Prog::AdjStages / Prog::AdjProg where the program has
// them, else the step's own.
template <class Prog, class = void>
struct AdjForward {
  template <class Own>
  static Own stages(Own o) { return o; }
  static constexpr int kMids = Prog::kMids;
};
template <class Prog>
struct AdjForward<Prog, std::void_t<typename Prog::AdjStages>> {
  template <class Own>
  static typename Prog::AdjStages stages(Own) { return {}; }
  static constexpr int kMids = Prog::AdjProg::kMids;
};

template <class Acc, class Rec, class List>
struct Recompute;
template <class Acc, class Rec, class... S>
struct Recompute<Acc, Rec, fgb::StageTypes<S...>> {
  static void run(Grid& g) {
    int s = 0;
    ((Rec::kStage[s++] ? sweep<Acc, S>(g) : void()), ...);
  }
};

template <class Prog, class... Stages>
struct Runner {
  using FwdAcc = Fwd<Prog::kDim, Prog::kShift>;
  using AF = AdjForward<Prog>;
  static void init(Grid& g, const int* n, const double* U) {
    for (int a = 0; a < 3; ++a) g.n[a] = 1;
    for (int a = 0; a < Prog::kDim; ++a) g.n[3 - Prog::kDim + a] = n[a];
    g.cells = (size_t)g.n[0] * g.n[1] * g.n[2];
    g.U = U;
    const int nm = Prog::kMids > AF::kMids ? Prog::kMids : AF::kMids;
    g.mids.assign((size_t)nm * g.cells + 1, 0.0);
  }
  static void forward(Grid& g, int upto) {   // stages [0, upto)
    int s = 0;
    ((s++ < upto ? sweep<FwdAcc, Stages>(g) : void()), ...);
  }
  template <class... Parts>
  static void partials(Grid& g, fgb::AdjParts<Parts...>) {
    (sweep<Partial, Parts>(g), ...);
  }
  template <class P>
  static void stage_pair(Grid& g, int& most) {
    if constexpr (P::P1::kDirect) {
      sweep<Direct<typename P::P1::Parts>, typename P::P2>(g);
    } else {
      g.pairs.assign((size_t)P::P1::kPairs * g.cells + 1, 0.0);
      partials(g, typename P::P1::Parts{});
      sweep<Gather, typename P::P2>(g);
    }
    (void)most;
  }
  template <class Rec, class... Pairs, class List>
  static void recompute_flags(Grid& g, fgb::AdjointStages<Rec, Pairs...>, List) {
    Recompute<FwdAcc, Rec, List>::run(g);
  }
  template <class Rec, class... Pairs, size_t... I>
  static void reverse_pairs(Grid& g, fgb::AdjointStages<Rec, Pairs...>, std::index_sequence<I...>) {
    using List = std::tuple<Pairs...>;
    int most = 0;
    constexpr size_t N = sizeof...(Pairs);
    (stage_pair<typename std::tuple_element<N - 1 - I, List>::type>(g, most), ...);
  }
  static int backward(Grid& g) {
    if constexpr (!std::is_same<typename Prog::Adjoint, void>::value) {
      sweep<Adj1, typename Prog::Adjoint>(g);
      return 0;
    } else if constexpr (!std::is_same<typename Prog::StageAdjoint, void>::value) {
      recompute_flags(g, typename Prog::StageAdjoint{}, AF::stages(fgb::StageTypes<Stages...>{}));
      g.lmids.assign((size_t)AF::kMids * g.cells + 1, 0.0);
      reverse_pairs(g, typename Prog::StageAdjoint{}, std::make_index_sequence<Prog::kStages>{});
      return 0;
    } else {
      return 1;
    }
  }
};

}  // namespace hostshim

#define FGB_DEFINE_PROGRAM(NAME, PROG, FIELDS, ...)                                                  \
  using hostshim_runner_##NAME = hostshim::Runner<PROG, __VA_ARGS__>;                                \
  extern "C" int host_forward_##NAME(const int* n, const double* U, const double* u, double* out) {  \
    hostshim::Grid g;                                                                                \
    hostshim_runner_##NAME::init(g, n, U);                                                           \
    g.u = u;                                                                                         \
    g.out = out;                                                                                     \
    hostshim_runner_##NAME::forward(g, PROG::kStages);                                               \
    return 0;                                                                                        \
  }                                                                                                  \
  extern "C" int host_backward_##NAME(const int* n, const double* U, const double* u,                \
                                      const double* lnext, double* lprev) {                          \
    hostshim::Grid g;                                                                                \
    hostshim_runner_##NAME::init(g, n, U);                                                           \
    g.u = u;                                                                                         \
    g.out = nullptr;                                                                                 \
    g.lnext = lnext;                                                                                 \
    g.lprev = lprev;                                                                                 \
    return hostshim_runner_##NAME::backward(g);                                                      \
  }
