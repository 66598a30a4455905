// CPU oracle for the BP-Layers hot path: a plain C++ restatement of the
// reference ops' arithmetic.  TEST INFRASTRUCTURE ONLY: it is linked by the
// tests, by the smoke check and by the benchmark's CPU-baseline leg, never by
// the product library.
//
// What it restates (paths relative to the reference project root):
//   * min-sum LBP forward, three pairwise variants
//       ops/lbp_stereo/src/lbp_min_sum_kernel.cu:9-213 (kernel), :424-500 (sweeps)
//       ops/lbp_stereo/src/util.cuh:103-118 (jump-tap index)
//       ops/lbp_semantic_pw/src/lbp_min_sum_kernel.cu:9-214
//       ops/lbp_semantic_pw_pixel/src/lbp_min_sum_kernel.cu:9-214
//   * the reference adjoint ("backward_minsum")
//       ops/lbp_stereo/src/lbp_min_sum_kernel.cu:215-417, :513-621
//       ops/lbp_stereo/src/util.cuh:9-85, :121-132
//       ops/lbp_semantic_pw/src/lbp_min_sum_kernel.cu:216-418 (pairwise grad :395-402)
//       ops/lbp_semantic_pw_pixel/src/lbp_min_sum_kernel.cu:216-417 (no edge grad)
//   * stereo SAD      ops/sad/src/stereo_sad_kernel.cu:16-108, :116-165
//   * flow MP-SAD     ops/flow_mp_sad/src/flow_mp_sad_kernel.cu:10-200, :208-290
//
// Two arithmetic modes for the LBP forward:
//   f32 : emulates the reference bit for bit: float adds in the reference's
//         order, fmaf where nvcc contracts `a + b*c`, the reference's
//         stride-halving tree for min/argmin and for the exp-sum, and
//         exp/log evaluated in double then rounded to float.
//         Build with -ffp-contract=off so the host compiler adds no FMAs.
//   f64 : the same recurrence in double (the "FP64 oracle"), used to state
//         the error of the FP32/FP16 kernels and for finite differences.
// The reference adjoint is evaluated with double accumulators in a fixed
// order (the reference itself uses float atomics in arbitrary order).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum { LEFT = 0, RIGHT = 1, UP = 2, DOWN = 3 };
enum { VAR_STEREO = 0, VAR_SEM_GLOBAL = 1, VAR_SEM_PIXEL = 2 };

inline int opposite(int d) { return d ^ 1; }

// float -> unsigned short as the reference's static_cast compiles on the GPU
// (PTX float-to-integer conversions clamp to the destination range; NaN -> 0).
inline int sat_u16(float v) {
  if (!(v > 0.0f)) return 0;
  if (v >= 65535.0f) return 65535;
  return static_cast<int>(v);
}

// power-of-two block width over labels used by the reference launch
// (lbp_min_sum_kernel.cu:445): min(2^ceil(log2 C), 1024)
inline int tree_width(int C) {
  int p = 1;
  while (p < C) p <<= 1;
  return std::min(p, 1024);
}

struct Shape {
  int B, H, W, L;
  int64_t pix(int n, int y, int x) const { return (static_cast<int64_t>(n) * H + y) * W + x; }
  // messages / argmin: (B,4,H,W,L)
  int64_t msg(int n, int d, int y, int x) const {
    return (((static_cast<int64_t>(n) * 4 + d) * H + y) * W + x) * L;
  }
  // scale / edge: (B,4,H,W)
  int64_t dir(int n, int d, int y, int x) const {
    return ((static_cast<int64_t>(n) * 4 + d) * H + y) * W + x;
  }
};

// Pairwise access for the three variants.
struct Pairwise {
  int variant;
  int Lv;         // stereo: number of jump taps (6 or 8)
  int jb;         // stereo: jump batch (1 or B)
  const void* j;  // float or double array, see T
};

template <typename T>
struct PairwiseT {
  int variant, Lv, jb, H, W, L;
  const T* j;
  // stereo taps: (Bj,4,Lv,H,W)
  T tap(int n, int d, int k, int y, int x) const {
    int nj = (jb == 1) ? 0 : n;
    return j[((((static_cast<int64_t>(nj) * 4 + d) * Lv + k) * H + y) * W + x)];
  }
  static int tap_index(int t, int s, int Lv) {
    int v = Lv / 2 + (t - s);
    v = std::max(1, v);
    v = std::min(Lv - 1, v);
    return v;
  }
  // f(t, s): cost of receiver label t given sender label s
  T f(int n, int d, int y, int x, int t, int s) const {
    switch (variant) {
      case VAR_STEREO: return tap(n, d, tap_index(t, s, Lv), y, x);
      case VAR_SEM_GLOBAL: return j[(static_cast<int64_t>(d) * L + s) * L + t];
      default: return j[((((static_cast<int64_t>(d) * H + y) * W + x) * L + s) * L + t)];
    }
  }
  T l2(int n, int d, int y, int x) const {
    switch (variant) {
      case VAR_STEREO: return tap(n, d, Lv - 1, y, x);
      case VAR_SEM_GLOBAL: return j[(static_cast<int64_t>(d) * L + 0) * L + (L - 1)];
      default: return j[((((static_cast<int64_t>(d) * H + y) * W + x) * L + 0) * L + (L - 1))];
    }
  }
};

inline float fma_t(float a, float b, float c) { return std::fmaf(a, b, c); }
inline double fma_t(double a, double b, double c) { return std::fma(a, b, c); }

// exp/log of the normalisation.  f32 mode: double evaluation rounded to float
// (lbp_min_sum_kernel.cu:167, :180-181).
inline float norm_exp(float m) { return static_cast<float>(std::exp(static_cast<double>(m))); }
inline double norm_exp(double m) { return std::exp(m); }

// One message step: sender pixel (n,y,x) in sweep direction d.
// Writes messages/argmin/scale at the receiver.  Scratch vectors are sized L.
template <typename T>
void lbp_step(const Shape& S, const PairwiseT<T>& P, const T* cost, const T* edge, int eb,
              T* msgs, float* argmin, T* scale, int delta, int n, int y, int x, int d,
              T* h, T* mval, int* marg, T* tv, float* tl) {
  const int C = S.L;
  const T* cst = cost + S.pix(n, y, x) * C;
  const T* mR = msgs + S.msg(n, RIGHT, y, x);
  const T* mL = msgs + S.msg(n, LEFT, y, x);
  const T* mU = msgs + S.msg(n, UP, y, x);
  const T* mD = msgs + S.msg(n, DOWN, y, x);
  for (int c = 0; c < C; ++c) {
    T v = cst[c];
    if (d != RIGHT) v += mR[c];
    if (d != LEFT) v += mL[c];
    if (d != UP) v += mU[c];
    if (d != DOWN) v += mD[c];
    h[c] = v;
  }
  const T w = edge[S.dir(eb == 1 ? 0 : n, d, y, x)];
  const int P2 = tree_width(C);
  const T max_float = static_cast<T>(1e15f);

  if (delta >= C) {
    // full min over all sender labels (lbp_min_sum_kernel.cu:88-111)
    for (int t = 0; t < C; ++t) {
      T msg = max_float;
      int am = 0;
      for (int s = 0; s < C; ++s) {
        T nm = fma_t(P.f(n, d, y, x, t, s), w, h[s]);
        msg = std::fmin(msg, nm);
        if (msg == nm) am = s;
      }
      mval[t] = msg;
      marg[t] = am;
    }
  } else {
    // truncated branch (lbp_min_sum_kernel.cu:112-164): tree argmin of h,
    // ties resolved towards the higher tree position (`<=`, :128)
    for (int c = 0; c < C; ++c) { tv[c] = h[c]; tl[c] = static_cast<float>(c); }
    for (int s = P2 / 2; s > 0; s >>= 1)
      for (int i = 0; i < s && i + s < C; ++i)
        if (tv[i + s] <= tv[i]) { tv[i] = tv[i + s]; tl[i] = tl[i + s]; }
    const T min_h = tv[0];
    const int argmin_h = static_cast<int>(tl[0]);
    const T L2 = P.l2(n, d, y, x);
    for (int t = 0; t < C; ++t) {
      T msg = fma_t(L2, w, min_h);
      int am = argmin_h;
      int start, stop;  // [start, stop)
      if (P.variant == VAR_STEREO) {
        const float off = static_cast<float>(P.tap(n, d, 0, y, x));
        start = sat_u16(std::round((static_cast<float>(t - (delta - 1)) + off) - 1.0f));
        stop = std::min(sat_u16(std::round((static_cast<float>(t + delta) + off) + 1.0f)), C);
      } else {
        start = std::max(t - delta + 1, 0);
        stop = std::min(t + delta - 1, C - 1) + 1;
      }
      for (int s = start; s < stop; ++s) {
        T nm = fma_t(P.f(n, d, y, x, t, s), w, h[s]);
        if (nm <= msg) { msg = nm; am = s; }
      }
      mval[t] = msg;
      marg[t] = am;
    }
  }

  // normalisation (lbp_min_sum_kernel.cu:166-181): exp, tree sum, log
  for (int c = 0; c < C; ++c) tv[c] = norm_exp(mval[c]);
  for (int s = P2 / 2; s > 0; s >>= 1)
    for (int i = 0; i < s && i + s < C; ++i) tv[i] += tv[i + s];
  double sum_exp = std::max(static_cast<double>(tv[0]), 1e-45);
  T lse = static_cast<T>(std::log(sum_exp));

  int qy = y, qx = x;
  if (d == RIGHT) qx = x + 1;
  if (d == LEFT) qx = x - 1;
  if (d == UP) qy = y - 1;
  if (d == DOWN) qy = y + 1;
  const int od = opposite(d);
  T* out = msgs + S.msg(n, od, qy, qx);
  float* oam = argmin ? argmin + S.msg(n, od, qy, qx) : nullptr;
  for (int c = 0; c < C; ++c) {
    out[c] = mval[c] - lse;
    if (oam) oam[c] = static_cast<float>(marg[c]);
  }
  scale[S.dir(n, od, qy, qx)] = static_cast<T>(sum_exp);
}

template <typename T>
void lbp_forward(int variant, const T* cost, const T* jump, const T* edge, T* msgs, float* argmin,
                 T* scale, int B, int H, int W, int L, int Lv, int jb, int eb, int delta,
                 int all_batches, int threads) {
  Shape S{B, H, W, L};
  PairwiseT<T> P{variant, Lv, jb, H, W, L, jump};
  const int nb = all_batches ? B : 1;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
  for (int n = 0; n < nb; ++n) {
    // sweep order of the reference host loop (lbp_min_sum_kernel.cu:461-491):
    // RIGHT, LEFT, DOWN, UP.  Rows (columns) of one sweep are independent.
    for (int d : {RIGHT, LEFT, DOWN, UP}) {
      const bool horiz = (d == RIGHT || d == LEFT);
      const int nchains = horiz ? H : W;
#pragma omp parallel
      {
        std::vector<T> h(L), mval(L), tv(L);
        std::vector<int> marg(L);
        std::vector<float> tl(L);
#pragma omp for schedule(dynamic, 1)
        for (int ch = 0; ch < nchains; ++ch) {
          if (d == RIGHT)
            for (int x = 0; x < W - 1; ++x)
              lbp_step(S, P, cost, edge, eb, msgs, argmin, scale, delta, n, ch, x, d, h.data(), mval.data(), marg.data(), tv.data(), tl.data());
          else if (d == LEFT)
            for (int x = W - 1; x > 0; --x)
              lbp_step(S, P, cost, edge, eb, msgs, argmin, scale, delta, n, ch, x, d, h.data(), mval.data(), marg.data(), tv.data(), tl.data());
          else if (d == DOWN)
            for (int y = 0; y < H - 1; ++y)
              lbp_step(S, P, cost, edge, eb, msgs, argmin, scale, delta, n, y, ch, d, h.data(), mval.data(), marg.data(), tv.data(), tl.data());
          else
            for (int y = H - 1; y > 0; --y)
              lbp_step(S, P, cost, edge, eb, msgs, argmin, scale, delta, n, y, ch, d, h.data(), mval.data(), marg.data(), tv.data(), tl.data());
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Reference adjoint (lbp_min_sum_kernel.cu:215-417, :513-621), double
// accumulation.  Reproduces the reference's structure, including what makes
// it differ from the exact gradient:
//   * grad_messages is in_grad passed through unchanged (:534-536);
//   * vertical sweeps carry no cross terms (compute_cross=false, :577, :587);
//   * horizontal sweeps add the saved vertical chain gradients of the
//     receiver (:380-386) without the normalisation Jacobian;
//   * the LSE Jacobian is taken from the messages/scale it is given.
// Pairwise-gradient layout per variant:
//   stereo  (B,4,Lv,H,W)   [reference allocates batch 1 and indexes by n]
//   global  (B,4,L,L)      [reference writes batch 0 only, :395-397]
//   pixel   (4,H,W,L,L)
// Edge gradient: (B,4,H,W) per batch item; pixel has none.
// Reference adjoint (exact = false) and exact adjoint (exact = true) of one
// pass.  The exact adjoint is the reverse-mode derivative of the forward
// pass as written: sweeps undone in reverse order (UP, DOWN, then LEFT,
// RIGHT; each orientation's two sweeps are independent), every step taking
// a = (upstream gradient of the message) + (gradients of its later readers)
// through J^T = I - p 1^T of the log normalisation and scattering it to h of
// the sender by argmin.  A horizontal message's later readers are the next
// step of its sweep (acc) and the two vertical sweeps at the receiver (the
// saved vertical accumulators); the reference instead carries the vertical
// parts as separate accumulators without J^T and returns in_grad as the
// message gradient (lbp_min_sum_kernel.cu:380-386, :534-536).  The exact
// message gradient is with respect to the pass's input messages: the old
// vertical messages read by the horizontal sweeps, the chain inputs at each
// sweep's first sender, and the upstream gradient of slots the pass never
// writes (those values pass through).
template <typename T>
void lbp_backward_t(int variant, bool exact, const T* jump, const T* edge, const T* in_grad,
                    const T* msgs, const float* argmin, const T* scale, double* g_cost,
                    double* g_jump, double* g_edge, double* g_msgs, int B, int H, int W, int L,
                    int Lv, int jb, int eb, int threads) {
  Shape S{B, H, W, L};
  PairwiseT<T> P{variant, Lv, jb, H, W, L, jump};
  const int64_t nmsg = static_cast<int64_t>(B) * 4 * H * W * L;
  if (!exact) {
    for (int64_t i = 0; i < nmsg; ++i) g_msgs[i] = in_grad[i];
  } else {
    for (int64_t i = 0; i < nmsg; ++i) g_msgs[i] = 0.0;
  }
  std::vector<double> saved(nmsg, 0.0);
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
  for (int n = 0; n < B; ++n) {
    // backward sweep order (:571-609): DOWN (undoes UP), UP (undoes DOWN),
    // LEFT (undoes RIGHT), RIGHT (undoes LEFT)
    for (int db : {DOWN, UP, LEFT, RIGHT}) {
      const int fd = opposite(db);  // forward direction = grad_xy_idx
      const bool horiz = (db == LEFT || db == RIGHT);
      const bool cross = horiz;
      const int nchains = horiz ? H : W;
      const int len = horiz ? W : H;
#pragma omp parallel
      {
        std::vector<double> acc(3 * L), nacc(3 * L), p(L), a(L);
        // the global-pairwise gradient is shared by every chain: accumulate
        // per thread, then reduce
        std::vector<double> gj_local(variant == VAR_SEM_GLOBAL ? static_cast<size_t>(L) * L : 0, 0.0);
#pragma omp for schedule(dynamic, 1)
        for (int ch = 0; ch < nchains; ++ch) {
          std::fill(acc.begin(), acc.end(), 0.0);
          int ly = 0, lx = 0;
          for (int k = 0; k < len - 1; ++k) {
            int y, x, qy, qx;
            if (db == DOWN) { x = ch; y = 1 + k; qy = y - 1; qx = x; }
            else if (db == UP) { x = ch; y = H - 2 - k; qy = y + 1; qx = x; }
            else if (db == LEFT) { y = ch; x = W - 2 - k; qy = y; qx = x + 1; }
            else { y = ch; x = 1 + k; qy = y; qx = x - 1; }
            ly = y;
            lx = x;
            const T* m = msgs + S.msg(n, db, qy, qx);
            const T* g = in_grad + S.msg(n, db, qy, qx);
            const float* am = argmin + S.msg(n, db, qy, qx);
            const double sc = scale[S.dir(n, db, qy, qx)];
            const double lsc = std::is_same<T, float>::value
                                   ? static_cast<double>(std::log(static_cast<float>(sc)))
                                   : std::log(sc);
            double sg = 0.0, sa = 0.0;
            for (int c = 0; c < L; ++c) {
              p[c] = std::exp(static_cast<double>(m[c]) + lsc) / sc;
              a[c] = g[c];
              if (exact && cross)
                a[c] += saved[S.msg(n, UP, qy, qx) + c] + saved[S.msg(n, DOWN, qy, qx) + c];
              sg += a[c];
              sa += acc[c];
            }
            const double w = edge[S.dir(eb == 1 ? 0 : n, fd, y, x)];
            std::fill(nacc.begin(), nacc.end(), 0.0);
            double ge = 0.0;
            for (int c = 0; c < L; ++c) {
              const double add_h = (a[c] - p[c] * sg) + (acc[c] - p[c] * sa);
              double add_u = 0.0, add_d = 0.0;
              if (cross && !exact) {
                add_u = saved[S.msg(n, UP, qy, qx) + c] + acc[L + c];
                add_d = saved[S.msg(n, DOWN, qy, qx) + c] + acc[2 * L + c];
              }
              const int s = static_cast<int>(am[c]);
              const double tot = add_h + add_u + add_d;
              g_cost[S.pix(n, y, x) * L + s] += tot;
              const double fv = P.f(n, fd, y, x, c, s);
              if (variant == VAR_STEREO) {
                const int k2 = PairwiseT<T>::tap_index(c, s, Lv);
                g_jump[((((static_cast<int64_t>(n) * 4 + fd) * Lv + k2) * H + y) * W + x)] += w * tot;
                ge += fv * tot;
              } else if (variant == VAR_SEM_GLOBAL) {
                gj_local[static_cast<size_t>(s) * L + c] += w * tot;
                ge += fv * tot;
              } else {
                g_jump[((((static_cast<int64_t>(fd) * H + y) * W + x) * L + s) * L + c)] += w * tot;
              }
              nacc[s] += add_h;
              nacc[L + s] += add_u;
              nacc[2 * L + s] += add_d;
            }
            // per batch item (the reference writes batch 0 for the global
            // variant, :400-402; identical at B=1, the only batch size its
            // forward processes)
            if (variant != VAR_SEM_PIXEL) g_edge[S.dir(n, fd, y, x)] += ge;
            acc.swap(nacc);
            double* sv = saved.data() + S.msg(n, db, y, x);
            for (int c = 0; c < L; ++c) sv[c] = acc[c];
            if (exact && cross) {
              // h of a horizontal sweep reads the pass's input vertical messages
              for (int c = 0; c < L; ++c) {
#pragma omp atomic
                g_msgs[S.msg(n, UP, y, x) + c] += acc[c];
#pragma omp atomic
                g_msgs[S.msg(n, DOWN, y, x) + c] += acc[c];
              }
            }
          }
          if (exact && len > 1) {
            // the chain input at the sweep's first sender (the last step here)
            double* gi = g_msgs + S.msg(n, db, ly, lx);
            for (int c = 0; c < L; ++c) {
#pragma omp atomic
              gi[c] += acc[c];
            }
          }
        }
        if (variant == VAR_SEM_GLOBAL) {
#pragma omp critical
          for (size_t i = 0; i < gj_local.size(); ++i)
            g_jump[(static_cast<int64_t>(0) * 4 + fd) * L * L + static_cast<int64_t>(i)] += gj_local[i];
        }
      }
    }
    if (exact) {
      // slots the pass never writes pass their input through: LEFT at x=0,
      // RIGHT at x=W-1, UP at y=0, DOWN at y=H-1; the vertical sweeps also
      // read the never-written horizontal ones
      for (int y = 0; y < H; ++y)
        for (int c = 0; c < L; ++c) {
          g_msgs[S.msg(n, LEFT, y, 0) + c] += in_grad[S.msg(n, LEFT, y, 0) + c] +
                                             saved[S.msg(n, UP, y, 0) + c] + saved[S.msg(n, DOWN, y, 0) + c];
          g_msgs[S.msg(n, RIGHT, y, W - 1) + c] += in_grad[S.msg(n, RIGHT, y, W - 1) + c] +
                                                  saved[S.msg(n, UP, y, W - 1) + c] +
                                                  saved[S.msg(n, DOWN, y, W - 1) + c];
        }
      for (int x = 0; x < W; ++x)
        for (int c = 0; c < L; ++c) {
          g_msgs[S.msg(n, UP, 0, x) + c] += in_grad[S.msg(n, UP, 0, x) + c];
          g_msgs[S.msg(n, DOWN, H - 1, x) + c] += in_grad[S.msg(n, DOWN, H - 1, x) + c];
        }
    }
  }
}

void lbp_backward_ref(int variant, const float* jump, const float* edge, const float* in_grad,
                      const float* msgs, const float* argmin, const float* scale, double* g_cost,
                      double* g_jump, double* g_edge, double* g_msgs, int B, int H, int W, int L,
                      int Lv, int jb, int eb, int threads) {
  lbp_backward_t<float>(variant, false, jump, edge, in_grad, msgs, argmin, scale, g_cost, g_jump, g_edge,
                        g_msgs, B, H, W, L, Lv, jb, eb, threads);
}

// ---------------------------------------------------------------------------
// Stereo SAD (ops/sad/src/stereo_sad_kernel.cu:16-108, :116-165)
void sad_forward(const float* f0, const float* f1, float* out, int B, int C, int H, int W,
                 int min_disp, int max_disp, float step, int all_batches, int threads) {
  const int D = static_cast<int>((max_disp - min_disp + 1) / step);
  const int64_t total = static_cast<int64_t>(B) * H * W * D;
  for (int64_t i = 0; i < total; ++i) out[i] = 40.0f;
  const int nb = all_batches ? B : 1;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
  for (int n = 0; n < nb; ++n) {
    const float* a = f0 + static_cast<int64_t>(n) * C * H * W;
    const float* b = f1 + static_cast<int64_t>(n) * C * H * W;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y) {
      for (int x = 0; x < W; ++x) {
        for (int di = 0; di < D; ++di) {
          const int d = static_cast<int>(static_cast<float>(di) * step + static_cast<float>(min_disp));
          const int xm = x - d;
          if (xm < 0 || xm >= W) continue;
          float sad = 0.0f;
          for (int c = 0; c < C; ++c) {
            const int64_t o = (static_cast<int64_t>(c) * H + y) * W;
            sad += std::fabs(a[o + x] - b[o + xm]);
          }
          out[((static_cast<int64_t>(n) * H + y) * W + x) * D + di] = sad;
        }
      }
    }
  }
}

// Backward (stereo_sad_kernel.cu:64-108).  `channel_limit` reproduces the
// reference launch covering only 4*ceil(D/4) channels (:152-157); pass C to
// cover all channels.
void sad_backward(const float* f0, const float* f1, const float* g, float* df0, float* df1, int B,
                  int C, int H, int W, int min_disp, int max_disp, int all_batches,
                  int channel_limit, int threads) {
  const int D = max_disp - min_disp + 1;
  const int64_t tot = static_cast<int64_t>(B) * C * H * W;
  std::memset(df0, 0, sizeof(float) * tot);
  std::memset(df1, 0, sizeof(float) * tot);
  const int nb = all_batches ? B : 1;
  const int cl = std::min(C, channel_limit);
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
  for (int n = 0; n < nb; ++n) {
    const float* a = f0 + static_cast<int64_t>(n) * C * H * W;
    const float* b = f1 + static_cast<int64_t>(n) * C * H * W;
    const float* gg = g + static_cast<int64_t>(n) * H * W * D;
    float* o0 = df0 + static_cast<int64_t>(n) * C * H * W;
    float* o1 = df1 + static_cast<int64_t>(n) * C * H * W;
#pragma omp parallel for schedule(static)
    for (int c = 0; c < cl; ++c) {
      for (int y = 0; y < H; ++y) {
        const int64_t o = (static_cast<int64_t>(c) * H + y) * W;
        for (int x = 0; x < W; ++x) {
          float g0 = 0.0f, g1 = 0.0f;
          for (int d = min_disp; d <= max_disp; ++d) {
            const int idx = d - min_disp;
            if (x - d >= 0 && x - d < W) {
              const float diff = a[o + x] - b[o + x - d];
              if (std::fabs(diff) > 1e-15f)
                g0 = std::fmaf(diff / std::fabs(diff), gg[(static_cast<int64_t>(y) * W + x) * D + idx], g0);
            }
            if (x + d >= 0 && x + d < W) {
              const float diff1 = a[o + x + d] - b[o + x];
              if (std::fabs(diff1) > 1e-15f)
                g1 = std::fmaf(-(diff1 / std::fabs(diff1)), gg[(static_cast<int64_t>(y) * W + x + d) * D + idx], g1);
            }
          }
          o0[o + x] = g0;
          o1[o + x] = g1;
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Flow max-projected SAD (ops/flow_mp_sad/src/flow_mp_sad_kernel.cu:10-124, :208-256)
void flow_forward(const float* f0, const float* f1, float* cv_u, float* cv_v, float* u_star,
                  float* v_star, int B, int C, int H, int W, int sws, int off_u, int off_v,
                  int blk_u, int blk_v, int all_batches, int threads) {
  const int K = sws + 1;
  const int hs = sws / 2;
  const int64_t tot = static_cast<int64_t>(B) * H * W * K;
  for (int64_t i = 0; i < tot; ++i) { cv_u[i] = 40.0f; cv_v[i] = 40.0f; u_star[i] = 0.0f; v_star[i] = 0.0f; }
  const int nb = all_batches ? B : 1;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
  for (int n = 0; n < nb; ++n) {
    const float* a = f0 + static_cast<int64_t>(n) * C * H * W;
    const float* b = f1 + static_cast<int64_t>(n) * C * H * W;
#pragma omp parallel
    {
      std::vector<float> win(static_cast<size_t>(K) * K);
#pragma omp for schedule(dynamic, 4)
      for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
          std::fill(win.begin(), win.end(), 40.0f);
          for (int ui = 0; ui < K; ++ui) {
            const int u = ui - hs;
            const int xm = x + off_u + u;
            if (xm < 0 || xm >= W) continue;
            for (int v = -hs; v <= hs; ++v) {
              const int vi = v + hs;
              const int ym = y + off_v + v;
              if (ym < 0 || ym >= H) continue;
              float sad = 0.0f;
              for (int c = 0; c < C; ++c)
                sad += std::fabs(a[(static_cast<int64_t>(c) * H + y) * W + x] - b[(static_cast<int64_t>(c) * H + ym) * W + xm]);
              win[static_cast<size_t>(vi) * K + ui] = sad;
            }
          }
          const int64_t o = ((static_cast<int64_t>(n) * H + y) * W + x) * K;
          for (int ui = 0; ui < K; ++ui) {
            float mn = 9999999.0f; int am = 0;
            for (int vi = 0; vi < K; ++vi)
              if (win[static_cast<size_t>(vi) * K + ui] < mn) { mn = win[static_cast<size_t>(vi) * K + ui]; am = vi; }
            cv_u[o + ui] = mn;
            u_star[o + ui] = static_cast<float>(am + blk_v * sws);
          }
          for (int vi = 0; vi < K; ++vi) {
            float mn = 9999999.0f; int am = 0;
            for (int ui = 0; ui < K; ++ui)
              if (win[static_cast<size_t>(vi) * K + ui] < mn) { mn = win[static_cast<size_t>(vi) * K + ui]; am = ui; }
            cv_v[o + vi] = mn;
            v_star[o + vi] = static_cast<float>(am + blk_u * sws);
          }
        }
      }
    }
  }
}

// Backward (flow_mp_sad_kernel.cu:126-200, :258-290); df1 accumulated in double
// in a fixed order (the reference uses float atomics).
void flow_backward(const float* f0, const float* f1, const float* gu, const float* gv,
                   const float* u_star, const float* v_star, float* df0, double* df1, int B, int C,
                   int H, int W, int sws, int all_batches) {
  const int hs = sws / 2;
  const int K = sws + 1;
  const int64_t tot = static_cast<int64_t>(B) * C * H * W;
  std::memset(df0, 0, sizeof(float) * tot);
  for (int64_t i = 0; i < tot; ++i) df1[i] = 0.0;
  const int nb = all_batches ? B : 1;
  for (int n = 0; n < nb; ++n) {
    const int64_t fo = static_cast<int64_t>(n) * C * H * W;
    for (int c = 0; c < C; ++c)
      for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
          const int64_t o = ((static_cast<int64_t>(n) * H + y) * W + x) * K;
          const float a = f0[fo + (static_cast<int64_t>(c) * H + y) * W + x];
          float g0 = 0.0f;
          for (int pass = 0; pass < 2; ++pass) {
            for (int i = -hs; i <= hs; ++i) {
              const int idx = i + hs;
              int u, v;
              if (pass == 0) { u = i; v = static_cast<int>(static_cast<short>(u_star[o + idx])) - hs; }
              else { v = i; u = static_cast<int>(static_cast<short>(v_star[o + idx])) - hs; }
              if (x + u >= 0 && x + u < W && y + v >= 0 && y + v < H) {
                const int64_t bi = fo + (static_cast<int64_t>(c) * H + y + v) * W + x + u;
                const float diff = a - f1[bi];
                if (std::fabs(diff) > 1e-15f) {
                  const float upd = diff / std::fabs(diff) * (pass == 0 ? gu[o + idx] : gv[o + idx]);
                  g0 += upd;
                  df1[bi] -= upd;
                }
              }
            }
          }
          df0[fo + (static_cast<int64_t>(c) * H + y) * W + x] = g0;
        }
  }
}

}  // namespace

extern "C" {

int oracle_version() { return 1; }

int oracle_max_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// LBP forward, float emulation of the reference.  argmin may be NULL.
void oracle_lbp_forward_f32(int variant, const float* cost, const float* jump, const float* edge,
                            float* messages, float* argmin, float* scale, int B, int H, int W,
                            int L, int Lv, int jump_batch, int edge_batch, int delta,
                            int all_batches, int threads) {
  lbp_forward<float>(variant, cost, jump, edge, messages, argmin, scale, B, H, W, L, Lv,
                     jump_batch, edge_batch, delta, all_batches, threads);
}

// LBP forward in double (FP64 oracle).
void oracle_lbp_forward_f64(int variant, const double* cost, const double* jump,
                            const double* edge, double* messages, float* argmin, double* scale,
                            int B, int H, int W, int L, int Lv, int jump_batch, int edge_batch,
                            int delta, int all_batches, int threads) {
  lbp_forward<double>(variant, cost, jump, edge, messages, argmin, scale, B, H, W, L, Lv,
                      jump_batch, edge_batch, delta, all_batches, threads);
}

void oracle_lbp_backward_ref(int variant, const float* jump, const float* edge,
                             const float* in_grad, const float* messages, const float* argmin,
                             const float* scale, double* grad_cost, double* grad_jump,
                             double* grad_edge, double* grad_messages, int B, int H, int W, int L,
                             int Lv, int jump_batch, int edge_batch, int threads) {
  lbp_backward_ref(variant, jump, edge, in_grad, messages, argmin, scale, grad_cost, grad_jump,
                   grad_edge, grad_messages, B, H, W, L, Lv, jump_batch, edge_batch, threads);
}

// Exact adjoint (see lbp_backward_t) for float and double forward results.
void oracle_lbp_backward_exact_f32(int variant, const float* jump, const float* edge,
                                   const float* in_grad, const float* messages, const float* argmin,
                                   const float* scale, double* grad_cost, double* grad_jump,
                                   double* grad_edge, double* grad_messages, int B, int H, int W,
                                   int L, int Lv, int jump_batch, int edge_batch, int threads) {
  lbp_backward_t<float>(variant, true, jump, edge, in_grad, messages, argmin, scale, grad_cost,
                        grad_jump, grad_edge, grad_messages, B, H, W, L, Lv, jump_batch, edge_batch,
                        threads);
}

void oracle_lbp_backward_exact_f64(int variant, const double* jump, const double* edge,
                                   const double* in_grad, const double* messages, const float* argmin,
                                   const double* scale, double* grad_cost, double* grad_jump,
                                   double* grad_edge, double* grad_messages, int B, int H, int W,
                                   int L, int Lv, int jump_batch, int edge_batch, int threads) {
  lbp_backward_t<double>(variant, true, jump, edge, in_grad, messages, argmin, scale, grad_cost,
                         grad_jump, grad_edge, grad_messages, B, H, W, L, Lv, jump_batch, edge_batch,
                         threads);
}

void oracle_sad_forward(const float* f0, const float* f1, float* out, int B, int C, int H, int W,
                        int min_disp, int max_disp, float step, int all_batches, int threads) {
  sad_forward(f0, f1, out, B, C, H, W, min_disp, max_disp, step, all_batches, threads);
}

void oracle_sad_backward(const float* f0, const float* f1, const float* g, float* df0, float* df1,
                         int B, int C, int H, int W, int min_disp, int max_disp, int all_batches,
                         int channel_limit, int threads) {
  sad_backward(f0, f1, g, df0, df1, B, C, H, W, min_disp, max_disp, all_batches, channel_limit,
               threads);
}

void oracle_flow_forward(const float* f0, const float* f1, float* cv_u, float* cv_v,
                         float* u_star, float* v_star, int B, int C, int H, int W, int sws,
                         int off_u, int off_v, int blk_u, int blk_v, int all_batches,
                         int threads) {
  flow_forward(f0, f1, cv_u, cv_v, u_star, v_star, B, C, H, W, sws, off_u, off_v, blk_u, blk_v,
               all_batches, threads);
}

void oracle_flow_backward(const float* f0, const float* f1, const float* gu, const float* gv,
                          const float* u_star, const float* v_star, float* df0, double* df1,
                          int B, int C, int H, int W, int sws, int all_batches) {
  flow_backward(f0, f1, gu, gv, u_star, v_star, df0, df1, B, C, H, W, sws, all_batches);
}

}  // extern "C"
