// Ghost-fill launches for sm_103a: the plain launch (one per TransferGroup),
// the fused stage launch's entry (its kernels instantiated in tam_fused_*.cu,
// one element type and dimension a unit), the solo groups (turned or
// bounded) and the arithmetic self-tests.  The kernels and what each item
// computes are in tam_kernels.cuh.
#include "tam_kernels.cuh"

namespace tam {

cudaError_t launch_plain_group(int dtype, int D, const DevGroup &g, const DevGroup *d_g,
                               const SchedArgs &a, void *work, const void *factors, int nvars,
                               const int S[3], cudaStream_t stream) {
  if (dtype == TAM_F64)
    return plain_dispatch<double>(D, g, d_g, typed<double>(a), (double *)work,
                                  (const double *)factors, nvars, S, stream);
  return plain_dispatch<float>(D, g, d_g, typed<float>(a), (float *)work, (const float *)factors,
                               nvars, S, stream);
}

cudaError_t launch_fused_stage(int dtype, int D, const Tile *tiles, const PTile *ptiles,
                               const Stage &st, const SchedArgs &a, void *work,
                               const void *factors, int nvars, const int S[3], int threads,
                               cudaStream_t stream, SideStream *side, const void *src,
                               const Tile *staged) {
  if (!src) src = work;
  ptiles += st.ptile0;
  staged += st.staged0;
  if (dtype != TAM_F64)
    return fused_stage_f32(D, tiles, ptiles, st, a, work, factors, nvars, S, threads, stream, side,
                           src, staged);
  switch (D) {
    case 1:
      return fused_stage_f64_d1(tiles, ptiles, st, a, work, factors, nvars, S, threads, stream,
                                side, src, staged);
    case 2:
      return fused_stage_f64_d2(tiles, ptiles, st, a, work, factors, nvars, S, threads, stream,
                                side, src, staged);
    default:
      return fused_stage_f64_d3(tiles, ptiles, st, a, work, factors, nvars, S, threads, stream,
                                side, src, staged);
  }
}

// ---- solo groups: turned across a seam, or bounded ------------------------------
// Julia's min and max of two floats (NaN-propagating, -0 below +0), which the
// bounded operators' extremes follow (src/ghosts.jl:291-361).
template <typename T>
__device__ __forceinline__ T jmin(T x, T y) {
  const bool c = (y < x) || (signbit(y) && !signbit(x));
  return c ? (isnan(x) ? x : y) : (isnan(y) ? y : x);
}
template <typename T>
__device__ __forceinline__ T jmax(T x, T y) {
  const bool c = (y > x) || (!signbit(y) && signbit(x));
  return c ? (isnan(x) ? x : y) : (isnan(y) ? y : x);
}
// minmod and the monotonized central slope (src/ghosts.jl:291-292)
template <typename T>
__device__ __forceinline__ T minmod(T a, T b) {
  return (a > T(0) && b > T(0)) ? jmin(a, b) : (a < T(0) && b < T(0)) ? jmax(a, b) : T(0);
}
template <typename T>
__device__ __forceinline__ T mc_slope(T a, T b) {
  using A = Arith<T>;
  return minmod(A::mul(T(2), a), minmod(A::mul(T(2), b), A::mul(A::add(a, b), T(0.5))));
}

// One item = (box point, variable, transfer) of solo group blockIdx.y.
// A turned group reads its real source through the axis map folded into
// signed strides: the virtual window's points are the real source's at
// c0 + sum_d vs[d] * j[d], variable rotvars[v + nvars * r] - 1
// (RotatedSource, src/ghosts.jl:183-244).  The sum is stencil_sum's
// (src/ghosts.jl:75-118): m_1 innermost, the weight product ((w_1*w_2)*w_3),
// acc from +0, no FMA, and with `one_tap` a dimension whose weight column has
// a single nonzero weight takes only that tap (src/ghosts.jl:28-56); a copy
// is +0 + x and a factor x*f + 0.  A bounded group computes bounded_sum
// (the parent at the order-3 window's middle row and its face neighbours,
// the monotonized central slopes, the child's side read off the stencil
// column, the largest scaling phi in [0, 1] that keeps every child within the
// extremes) or bracket_clamp_sum (the full order-p sum clamped into the
// range of the points with a nonzero linear weight in every dimension),
// each carrying 0 * (max - min) (src/ghosts.jl:291-361).  In a batch of
// forests the group's member gives the arrays' offsets in the arena and the
// stored extents; its odd turns read its own array.
template <typename T, int D>
__global__ void __launch_bounds__(256)
    solo_group_kernel(const SoloGroup *__restrict__ turns, Args<T> a, const T *src,
                      const T *alt, T *work, const T *__restrict__ factors,
                      const int32_t *__restrict__ rotvars, int nvars, int S1, int S2, int S3,
                      int32_t *err) {
  using A = Arith<T>;
  const SoloGroup tg = turns[blockIdx.y];
  const DevGroup &g = a.groups[tg.group];
  if (a.members) {
    const Member &m = a.members[g.member];
    src += m.work_off;
    alt = src;
    work += m.work_off;
    if (factors) factors += m.fac_off;
    S1 = m.S[0];
    S2 = m.S[1];
    S3 = m.S[2];
  }
  const int64_t box = (int64_t)g.n[0] * g.n[1] * g.n[2];
  const int64_t items = box * nvars * g.ntransfers;
  const int64_t vol = (int64_t)S1 * S2 * S3;
  const T *from = tg.odd ? alt : src;
  for (int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; it < items;
       it += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = it;
    const int i1 = (int)(r % g.n[0]);
    r /= g.n[0];
    const int i2 = (int)(r % g.n[1]);
    r /= g.n[1];
    const int i3 = (int)(r % g.n[2]);
    r /= g.n[2];
    const int v = (int)(r % nvars);
    const int64_t t = r / nvars + g.first;
    const int64_t tblock = __ldg(a.tb + t) - 1;
    const int64_t sblock = __ldg(a.sb + t) - 1;
    int sv = v;
    if (tg.col) {
      sv = __ldg(rotvars + v + (int64_t)nvars * tg.col) - 1;
      if (sv < 0 || sv >= nvars) {  // a variable table naming no variable: skip, and say so
        atomicExch(err, (int32_t)TAM_EINVAL);
        continue;
      }
    }
    const T *sp = from + (sblock * nvars + sv) * vol + tg.c0;
    const int idx[3] = {i1, i2, i3};
    int64_t j[3];
    int lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
    const T *wc[3];
    for (int k = 0; k < 3; ++k) {
      j[k] = __ldg(a.srcstart + g.ss[k] + idx[k]) - 1;
      wc[k] = a.weights + g.w[k] + (int64_t)g.order[k] * idx[k];
      hi[k] = (tg.bounded == 2 && k < D) ? g.order[k] / 2 : g.order[k];
      if (a.one_tap && k < D && !tg.bounded) {
        int nonzero = 0, row = 0;
        for (int m = 0; m < g.order[k]; ++m)
          if (wc[k][m] != T(0)) {
            ++nonzero;
            row = m;
          }
        if (nonzero == 1) {
          lo[k] = row;
          hi[k] = row + 1;
        }
      }
    }
    const int64_t vs0 = tg.vs[0], vs1 = tg.vs[1], vs2 = tg.vs[2];
    T x;
    if (tg.bounded == 1) {
      // bounded_sum: the parent at the window's middle row
      int64_t c[3] = {j[0], j[1], j[2]};
      for (int k = 0; k < D; ++k) c[k] += 1;
      const int64_t o = vs0 * c[0] + vs1 * c[1] + vs2 * c[2];
      const int64_t st[3] = {vs0, vs1, vs2};
      const T u = sp[o];
      T M = u, m = u, dl = T(0), sl = T(0);
      T lov[3], hiv[3], s[3];
      for (int k = 0; k < D; ++k) {
        lov[k] = sp[o - st[k]];
        hiv[k] = sp[o + st[k]];
        s[k] = mc_slope(A::add(hiv[k], -u), A::add(u, -lov[k]));
      }
      for (int k = 0; k < D; ++k) M = jmax(M, lov[k]);
      for (int k = 0; k < D; ++k) M = jmax(M, hiv[k]);
      for (int k = 0; k < D; ++k) m = jmin(m, lov[k]);
      for (int k = 0; k < D; ++k) m = jmin(m, hiv[k]);
      // the sums are right folds, t_1 + (t_2 + t_3)
      for (int k = D - 1; k >= 0; --k) {
        const T sg = wc[k][2] > wc[k][0] ? s[k] : -s[k];
        dl = k == D - 1 ? sg : A::add(sg, dl);
        const T as = fabs(s[k]);
        sl = k == D - 1 ? as : A::add(as, sl);
      }
      dl = A::mul(dl, T(0.25));
      sl = A::mul(sl, T(0.25));
      T phi = T(1);
      if (sl > T(0)) phi = jmin(jmin(T(1), (M - u) / sl), (u - m) / sl);
      x = A::add(A::add(u, A::mul(phi, dl)), A::mul(T(0), A::add(M, -m)));
    } else if (g.unit) {
      x = A::add(T(0), sp[vs0 * j[0] + vs1 * j[1] + vs2 * j[2]]);
    } else {
      T acc = T(0);
      T blo = T(INFINITY), bhi = T(-INFINITY);
      for (int m3 = lo[2]; m3 < hi[2]; ++m3)
        for (int m2 = lo[1]; m2 < hi[1]; ++m2)
          for (int m1 = lo[0]; m1 < hi[0]; ++m1) {
            T w = wc[0][m1];
            if (D >= 2) w = A::mul(w, wc[1][m2]);
            if (D >= 3) w = A::mul(w, wc[2][m3]);
            const T u = sp[vs0 * (j[0] + m1) + vs1 * (j[1] + m2) + vs2 * (j[2] + m3)];
            acc = A::add(acc, A::mul(w, u));
            if (tg.bounded == 2) {
              // the bracket: a nonzero linear weight in every dimension
              const bool in = wc[0][hi[0] + m1] != T(0) &&
                              (D < 2 || wc[1][hi[1] + m2] != T(0)) &&
                              (D < 3 || wc[2][hi[2] + m3] != T(0));
              if (in) {
                blo = jmin(blo, u);
                bhi = jmax(bhi, u);
              }
            }
          }
      x = acc;
      if (tg.bounded == 2) {
        const T cl = acc > bhi ? bhi : acc < blo ? blo : acc;
        x = A::add(cl, A::mul(T(0), A::add(bhi, -blo)));
      }
    }
    const int64_t toff = (tblock * nvars + v) * vol +
                         ((int64_t)(g.tf[2] + i3) * S2 + (g.tf[1] + i2)) * S1 + g.tf[0] + i1;
    work[toff] = scaled(x, factors, v, nvars, g.factorcol);
  }
}

template <typename T>
cudaError_t solo_dispatch(int D, const SoloGroup *turns, int64_t n, const Args<T> &a,
                            const T *src, const T *alt, T *work, const T *factors,
                            const int32_t *rotvars, int nvars, const int S[3], int32_t *err,
                            cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  // items of the largest turned group are not known here: a grid-stride
  // loop over a fixed x extent per group
  const dim3 grid(64, (unsigned)n), block(256);
  switch (D) {
    case 1:
      solo_group_kernel<T, 1><<<grid, block, 0, stream>>>(turns, a, src, alt, work, factors,
                                                             rotvars, nvars, S[0], S[1], S[2], err);
      break;
    case 2:
      solo_group_kernel<T, 2><<<grid, block, 0, stream>>>(turns, a, src, alt, work, factors,
                                                             rotvars, nvars, S[0], S[1], S[2], err);
      break;
    default:
      solo_group_kernel<T, 3><<<grid, block, 0, stream>>>(turns, a, src, alt, work, factors,
                                                             rotvars, nvars, S[0], S[1], S[2], err);
      break;
  }
  return cudaGetLastError();
}

cudaError_t launch_solo(int dtype, int D, const SoloGroup *turns, int64_t n,
                          const SchedArgs &a, const void *src, const void *alt, void *work,
                          const void *factors, const int32_t *rotvars, int nvars,
                          const int S[3], int32_t *err, cudaStream_t stream) {
  if (!alt) alt = src;
  if (dtype == TAM_F64)
    return solo_dispatch<double>(D, turns, n, typed<double>(a), (const double *)src,
                                   (const double *)alt, (double *)work, (const double *)factors,
                                   rotvars, nvars, S, err, stream);
  return solo_dispatch<float>(D, turns, n, typed<float>(a), (const float *)src,
                                (const float *)alt, (float *)work, (const float *)factors,
                                rotvars, nvars, S, err, stream);
}

std::vector<uint64_t> short_weights(const std::vector<unsigned char> &wtab) {
  std::vector<uint64_t> out(wtab.size() / 8);
  for (size_t i = 0; i < out.size(); ++i) {
    uint64_t b;
    memcpy(&b, wtab.data() + 8 * i, 8);
    const uint32_t whi = (uint32_t)(b >> 32), wlo = (uint32_t)b;
    const uint32_t wm = (((whi & 0xFFFFFu) | 0x100000u) << 3) | (wlo >> 29);
    const int ew = (int)((whi >> 20) & 0x7FF);
    const int we = ew == 0 ? -4096 : ew - 1023;   // as short_weight: a zero is flagged
    const uint32_t hi = (whi & 0x80000000u) | (uint32_t)(we + 8192);
    out[i] = ((uint64_t)hi << 32) | wm;
  }
  return out;
}

void pack_tiles(const std::vector<Tile> &tiles, const std::vector<uint16_t> *keys,
                int64_t begin, int64_t end, int target, std::vector<PTile> &out) {
  int64_t i = begin;
  while (i < end) {
    PTile p{(int32_t)i, 0, 0, 0};
    while (i < end && p.nseg < 32 &&
           (p.nseg == 0 || (p.nitems + tiles[i].nitems <= target &&
                            (!keys || (*keys)[i] == (*keys)[p.seg0])))) {
      p.nitems += tiles[i].nitems;
      ++p.nseg;
      ++i;
    }
    out.push_back(p);
  }
}

std::vector<PTile> pack_stages(std::vector<Stage> &stages, const std::vector<Tile> &tiles,
                               int target, const std::vector<uint16_t> *keys,
                               int stencil_target) {
  const int ts = stencil_target > 0 ? stencil_target : target;
  std::vector<PTile> out;
  for (Stage &st : stages) {
    st.ptile0 = (int64_t)out.size();
    pack_tiles(tiles, keys, st.tile0, st.tile0 + st.ncopy0, target, out);
    st.npcopy0 = (int64_t)out.size() - st.ptile0;
    pack_tiles(tiles, keys, st.tile0 + st.ncopy0, st.tile0 + st.ncopy, target, out);
    st.npcopy = (int64_t)out.size() - st.ptile0;
    // the stencils: with keys (tiles by path, sorted by key) the order-4
    // run packed on its own, so that its packed tiles are a run too
    int64_t b4 = st.tile0 + st.ncopy, e4 = b4;
    const int64_t send = st.tile0 + st.ncopy + st.nsten;
    if (keys) {
      auto four = [&](int64_t t) { return ((*keys)[t] >> 4) == 4 + 2; };
      while (b4 < send && !four(b4) && (*keys)[b4] < ((4 + 2) << 4)) ++b4;
      e4 = b4;
      while (e4 < send && four(e4)) ++e4;
    }
    pack_tiles(tiles, keys, st.tile0 + st.ncopy, b4, ts, out);
    st.np4_0 = (int64_t)out.size() - st.ptile0;
    pack_tiles(tiles, keys, b4, e4, ts, out);
    st.np4 = (int64_t)out.size() - st.ptile0 - st.np4_0;
    pack_tiles(tiles, keys, e4, send, ts, out);
    st.nptiles = (int64_t)out.size() - st.ptile0;
  }
  return out;
}

void StencilRuns::of(const DevGroup &g, const int32_t *csingle, const int32_t *perm, int D,
                     std::vector<Run> &runs) {
  runs.clear();
  const int box = g.n[0] * g.n[1] * g.n[2];
  const int base = (g.pclass + 2) << 4;
  auto mask_of = [&](int k) {
    if (g.perm < 0) return 8;
    const int p = perm[g.perm + k];
    const int idx[3] = {p % g.n[0], (p / g.n[0]) % g.n[1], p / (g.n[0] * g.n[1])};
    int m = 0;
    for (int d = 0; d < D; ++d)
      if (csingle[g.csingle[d] + idx[d]] >= 0) m |= 1 << d;
    return m;
  };
  int i0 = 0;
  while (i0 < box) {
    const int m = mask_of(i0);
    int i1 = i0 + 1;
    while (i1 < box && mask_of(i1) == m) ++i1;
    runs.push_back({i0, i1 - i0, (uint16_t)(base | m)});
    i0 = i1;
  }
}

void StencilRuns::tiles(int32_t gi, int32_t transfer, int ti, std::vector<Tile> &out,
                        std::vector<uint16_t> &keys) {
  const std::vector<Run> &runs = cache[gi];
  for (const Run &r : runs)
    for (int i0 = r.first; i0 < r.first + r.n; i0 += ti) {
      out.push_back({gi, transfer, i0, std::min(ti, r.first + r.n - i0)});
      keys.push_back(r.key);
    }
}

cudaError_t side_create(SideStream &s) {
  cudaError_t e = cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.join, cudaEventDisableTiming);
  if (e != cudaSuccess) side_destroy(s);
  return e;
}

void side_destroy(SideStream &s) {
  if (s.fork) cudaEventDestroy(s.fork);
  if (s.join) cudaEventDestroy(s.join);
  if (s.stream) cudaStreamDestroy(s.stream);
  s = SideStream{};
}

}  // namespace tam

// ---- self-test of the integer-pipe multiply ----------------------------------
namespace tam {
namespace {

__device__ __forceinline__ uint64_t splitmix(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Compares mul_short with __dmul_rn on n pseudo-random pairs: weights with
// random 24-bit significands, signs and exponents in [-40, 40]; data drawn
// from every bit pattern (specials, subnormals, extreme exponents) or, for
// half the pairs, near the weights' scale.  Counts bitwise differences, every
// NaN one pattern.
__global__ void selftest_mul_kernel(int64_t n, uint64_t seed,
                                    unsigned long long *__restrict__ mismatches) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t r1 = splitmix(seed ^ (uint64_t)(2 * i));
    const uint64_t r2 = splitmix(seed ^ (uint64_t)(2 * i + 1));
    // weight: sign, exponent in [-40, 40], 24-bit significand
    const uint64_t wexp = (uint64_t)(1023 - 40 + (int)(r1 % 81));
    const uint64_t wsig = (r1 >> 8) & 0x7FFFFFull;  // 23 fraction bits
    const uint64_t wbits = ((r1 >> 63) << 63) | (wexp << 52) | (wsig << 29);
    uint64_t ubits = r2;
    if (r1 & 0x100) {  // near the normal range's middle, and at its edges
      const uint64_t e = (r1 & 0x200) ? (uint64_t)(1 + (int)((r1 >> 10) % 60))
                                      : (uint64_t)(900 + (int)((r1 >> 10) % 250));
      ubits = (r2 & 0x800FFFFFFFFFFFFFull) | (e << 52);
    }
    const double w = __longlong_as_double((long long)wbits);
    const double u = __longlong_as_double((long long)ubits);
    const ShortW sw = short_weight(w);
    const double a = mul_short(sw.w, sw.wm, sw.we, sw.wsign, u);
    const double b = __dmul_rn(w, u);
    const bool same = (__double_as_longlong(a) == __double_as_longlong(b)) ||
                      (a != a && b != b);
    if (!same) atomicAdd(mismatches, 1ull);
  }
}

// add_soft against __dadd_rn: a the running sum (any sign and exponent,
// zeros, subnormals and specials among them), b a normal nonzero product at
// a distance from a that favours the adder's cases: equal exponents, one
// apart, cancellations (b near -a), far apart, and sums at the edges of the
// normal range.  A result the adder flags is not compared (the caller sums
// that point on the FP64 pipe); mismatches[1] counts them.
__global__ void selftest_add_kernel(int64_t n, uint64_t seed,
                                    unsigned long long *__restrict__ mismatches) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t r1 = splitmix(seed ^ (uint64_t)(3 * i));
    const uint64_t r2 = splitmix(seed ^ (uint64_t)(3 * i + 1));
    const uint64_t r3 = splitmix(seed ^ (uint64_t)(3 * i + 2));
    uint64_t abits = r1;
    const int mode = (int)(r3 & 7);
    if (mode < 6) {  // a normal a, exponent in the middle or near an edge
      const int ea = (r3 & 8) ? 1 + (int)((r3 >> 8) % 80)
                              : (r3 & 16) ? 1940 + (int)((r3 >> 8) % 107)
                                          : 900 + (int)((r3 >> 8) % 250);
      abits = (r1 & 0x800FFFFFFFFFFFFFull) | ((uint64_t)ea << 52);
    } else if (mode == 6) {  // a zero or a subnormal
      abits = (r1 & 0x8000000000000000ull) | ((r3 & 32) ? 0 : (r1 & 0x000FFFFFFFFFFFFFull));
    }
    const int eA = (int)((abits >> 52) & 0x7FF);
    // b's exponent: a's plus a distance, mostly small
    const int sel = (int)((r3 >> 20) & 15);
    int dist = sel < 4 ? 0 : sel < 7 ? 1 : sel < 9 ? -1 : sel < 11 ? 2 : sel < 12 ? -2
                                       : (int)((r3 >> 24) % 121) - 60;
    int eb = (eA == 0 ? 1 + (int)((r3 >> 24) % 2000) : eA) + dist;
    eb = eb < 1 ? 1 : eb > 2046 ? 2046 : eb;
    uint64_t bbits = (r2 & 0x800FFFFFFFFFFFFFull) | ((uint64_t)eb << 52);
    if (((r3 >> 32) & 3) == 0 && eA > 0 && eA < 2047) {
      // near -a: a's bits with the sign flipped and the low bits changed
      bbits = (abits ^ 0x8000000000000000ull) ^ (r2 & ((1ull << ((r3 >> 40) % 53)) - 1));
    }
    const double a = __longlong_as_double((long long)abits);
    const double b = __longlong_as_double((long long)bbits);
    const int be = (int)((bbits >> 52) & 0x7FF);
    if (be == 0 || be == 0x7FF) continue;  // b is a product of the fast path
    bool bad = false;
    const double s = add_soft(a, b, bad);
    if (bad) {
      atomicAdd(mismatches + 1, 1ull);
      continue;
    }
    const double t = __dadd_rn(a, b);
    if (__double_as_longlong(s) != __double_as_longlong(t)) atomicAdd(mismatches, 1ull);
  }
}

// mul_full against __dmul_rn: both factors of any sign and significand,
// exponents across the normal range and pairs whose product lands near its
// edges.  A product the multiply flags is not compared; mismatches[1]
// counts them.
__global__ void selftest_mul_full_kernel(int64_t n, uint64_t seed,
                                         unsigned long long *__restrict__ mismatches) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t r1 = splitmix(seed ^ (uint64_t)(3 * i));
    const uint64_t r2 = splitmix(seed ^ (uint64_t)(3 * i + 1));
    const uint64_t r3 = splitmix(seed ^ (uint64_t)(3 * i + 2));
    const int ew = 1 + (int)((r3 & 0xFFFF) % 2046);
    int eu;
    switch ((r3 >> 16) & 3) {
      case 0: eu = 1 + (int)((r3 >> 20) % 2046); break;          // anywhere
      case 1: eu = 2046 + 1023 - ew + (int)((r3 >> 20) % 7) - 3; break;  // near overflow
      case 2: eu = 1023 + 1 - ew + (int)((r3 >> 20) % 64) - 3; break;   // near underflow
      default: eu = 2046 - ew + (int)((r3 >> 20) % 41) - 20; break;      // mid-range
    }
    eu = eu < 1 ? 1 : eu > 2046 ? 2046 : eu;
    const uint64_t wb = (r1 & 0x800FFFFFFFFFFFFFull) | ((uint64_t)ew << 52);
    const uint64_t ub = (r2 & 0x800FFFFFFFFFFFFFull) | ((uint64_t)eu << 52);
    const double w = __longlong_as_double((long long)wb);
    const double u = __longlong_as_double((long long)ub);
    bool bad = false;
    const double p = mul_full(w, u, bad);
    if (bad) {
      atomicAdd(mismatches + 1, 1ull);
      continue;
    }
    if (__double_as_longlong(p) != __double_as_longlong(__dmul_rn(w, u)))
      atomicAdd(mismatches, 1ull);
  }
}

}  // namespace

cudaError_t launch_selftest_mul_full(int64_t n, uint64_t seed, unsigned long long *mismatches,
                                     cudaStream_t stream) {
  selftest_mul_full_kernel<<<1216, 256, 0, stream>>>(n, seed, mismatches);
  return cudaGetLastError();
}

cudaError_t launch_selftest_mul(int64_t n, uint64_t seed, unsigned long long *mismatches,
                                cudaStream_t stream) {
  selftest_mul_kernel<<<1216, 256, 0, stream>>>(n, seed, mismatches);
  return cudaGetLastError();
}

cudaError_t launch_selftest_add(int64_t n, uint64_t seed, unsigned long long *mismatches,
                                cudaStream_t stream) {
  selftest_add_kernel<<<1216, 256, 0, stream>>>(n, seed, mismatches);
  return cudaGetLastError();
}

}  // namespace tam
