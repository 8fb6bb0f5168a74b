// Host checks of the device arithmetic that the mixed path is built on,
// compiled from the same headers as the kernels (ttg_df64.cuh,
// ttg_gemm_live.h):
//   * df_split_pow2 / f32_to_f64_pow2 / df_join_pow2 -- the bit-level FP64 <->
//     double-float conversions with a power-of-two scale: normalisation
//     (|lo| <= ulp(hi)/2), accuracy (2^-48 of |x 2^k| where lo is kept),
//     round trips, signed zeros, infinities, NaN, the flush thresholds and
//     the rounding carry out of the significand;
//   * df_add / df_mul / df_fma against long double, within the double-word
//     error bounds of Joldes, Muller & Popescu (ACM TOMS 2017: 3u^2 for
//     DWPlusDW, 5u^2 for DWTimesDW with FMA; u = 2^-24), and the sum of
//     the product's and the sum's bounds for the fused form;
//   * df_recip and df_sqrt (one Newton step each) against long double;
//   * gemm_live, the per-thread live-row rule of the GEMM tiles, against a
//     brute-force enumeration of every product a tile must form.
// Prints "OK" and exits 0 when every check passes.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <random>

#include "ttg_df64.cuh"
#include "ttg_gemm_live.h"

using ttg::df64;

static int g_fail = 0;
#define CHECK(cond, ...)                    \
  do                                        \
  {                                         \
    if (!(cond))                            \
    {                                       \
      if (g_fail < 20)                      \
      {                                     \
        std::printf("FAIL %s: ", #cond);    \
        std::printf(__VA_ARGS__);           \
        std::printf("\n");                  \
      }                                     \
      ++g_fail;                             \
    }                                       \
  } while (0)

static long double pair_value(df64 a) { return static_cast<long double>(a.hi) + a.lo; }

static void check_split()
{
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::uniform_int_distribution<int> ek(-60, 60), kk(-40, 40);
  double worst = 0.0, worst_rt = 0.0;
  for (int it = 0; it < 400000; ++it)
  {
    const double x = std::ldexp(u(rng), ek(rng));
    const int k = kk(rng);
    const long double xs = std::ldexp(static_cast<long double>(x), k);
    const df64 p = ttg::df_split_pow2(x, k);
    if (x == 0.0 || std::fabs(static_cast<double>(xs)) < 0x1p-126 ||
        std::fabs(static_cast<double>(xs)) >= 0x1p127)
      continue;
    // normalised pair: hi is xs rounded to 24 bits, |lo| <= ulp(hi) / 2
    const double ulp = std::ldexp(1.0, std::ilogb(p.hi) - 23);
    CHECK(std::fabs(p.lo) <= 0.5 * ulp, "x=%a k=%d hi=%a lo=%a", x, k, p.hi, p.lo);
    const bool lo_kept = std::fabs(static_cast<double>(xs)) >= 0x1p-74;
    const double err = static_cast<double>(std::fabs(pair_value(p) - xs) / std::fabs(xs));
    if (lo_kept)
    {
      worst = std::fmax(worst, err);
      CHECK(err <= 0x1p-48, "x=%a k=%d err=%g", x, k, err);
      // back to FP64 with the inverse scale: within 2^-48 (lo's rounding)
      const double y = ttg::df_join_pow2(p, -k);
      const double rt = std::fabs(y - x) / std::fabs(x);
      worst_rt = std::fmax(worst_rt, rt);
      CHECK(rt <= 0x1p-47, "round trip x=%a k=%d y=%a", x, k, y);
    }
    else
      CHECK(err <= 0x1p-23, "flushed lo x=%a k=%d err=%g", x, k, err);
  }
  std::printf("split: worst rel. err %.3g (2^-48 = %.3g), round trip %.3g\n", worst, 0x1p-48,
              worst_rt);
  // special values
  df64 z = ttg::df_split_pow2(0.0, 5);
  CHECK(z.hi == 0.0f && !std::signbit(z.hi) && z.lo == 0.0f, "+0");
  z = ttg::df_split_pow2(-0.0, 5);
  CHECK(z.hi == 0.0f && std::signbit(z.hi), "-0");
  z = ttg::df_split_pow2(INFINITY, 0);
  CHECK(std::isinf(z.hi) && z.hi > 0, "+inf");
  z = ttg::df_split_pow2(-INFINITY, 3);
  CHECK(std::isinf(z.hi) && z.hi < 0, "-inf");
  z = ttg::df_split_pow2(NAN, 0);
  CHECK(std::isnan(z.hi), "nan");
  z = ttg::df_split_pow2(1.0, 200);  // beyond the float range
  CHECK(std::isinf(z.hi), "overflow to inf");
  z = ttg::df_split_pow2(1.0, -127);  // below 2^-126: flushed
  CHECK(z.hi == 0.0f && z.lo == 0.0f, "flush to zero");
  z = ttg::df_split_pow2(5e-324, 0);  // subnormal double
  CHECK(z.hi == 0.0f, "subnormal input");
  // rounding carry: 2 - 2^-52 rounds hi up to 2.0 with a negative lo
  z = ttg::df_split_pow2(2.0 - 0x1p-52, 0);
  CHECK(z.hi == 2.0f && z.lo == -0x1p-52f, "carry hi=%a lo=%a", z.hi, z.lo);
  z = ttg::df_split_pow2(-(2.0 - 0x1p-52), 1);
  CHECK(z.hi == -4.0f && z.lo == 0x1p-51f, "negative carry hi=%a lo=%a", z.hi, z.lo);
  // exact for 24-bit values, scale folded into the exponent
  z = ttg::df_split_pow2(3.0, -2);
  CHECK(z.hi == 0.75f && z.lo == 0.0f, "exact 3/4");
  CHECK(ttg::pow2_exponent(0x1p-7) == -7 && ttg::pow2_exponent(1.0) == 0 &&
          ttg::pow2_exponent(0x1p30) == 30,
        "pow2_exponent");
  // f32 -> f64 conversion: exact for normal floats, flush / inf / nan
  CHECK(ttg::f32_to_f64_pow2(1.5f, 3) == 12.0, "f32 scale");
  CHECK(ttg::f32_to_f64_pow2(-0x1.fffffep127f, 0) == -0x1.fffffep127, "f32 max");
  CHECK(ttg::f32_to_f64_pow2(0x1p-149f, 0) == 0.0, "subnormal float flushes");
  CHECK(std::isinf(ttg::f32_to_f64_pow2(INFINITY, 0)), "inf");
  CHECK(std::isnan(ttg::f32_to_f64_pow2(NAN, 0)), "nan");
  CHECK(std::isinf(ttg::f32_to_f64_pow2(1.0f, 1100)), "f64 overflow");
}

static df64 random_pair(std::mt19937_64& rng)
{
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::uniform_int_distribution<int> ek(-20, 20);
  return ttg::df_split_pow2(std::ldexp(u(rng), ek(rng)), 0);
}

static void check_ops()
{
  const long double u = 0x1p-24L;
  std::mt19937_64 rng(5);
  double wa = 0.0, wm = 0.0, wf = 0.0;
  for (int it = 0; it < 300000; ++it)
  {
    const df64 a = random_pair(rng), b = random_pair(rng), c = random_pair(rng);
    const long double av = pair_value(a), bv = pair_value(b), cv = pair_value(c);
    const long double s = av + bv, p = av * bv, f = av * bv + cv;
    if (s != 0.0L)
    {
      const long double e = std::fabs(pair_value(ttg::df_add(a, b)) - s) / std::fabs(s);
      wa = std::fmax(wa, static_cast<double>(e / (u * u)));
      CHECK(e <= 3 * u * u, "df_add err %Lg u^2", e / (u * u));
    }
    if (p != 0.0L)
    {
      const long double e = std::fabs(pair_value(ttg::df_mul(a, b)) - p) / std::fabs(p);
      wm = std::fmax(wm, static_cast<double>(e / (u * u)));
      CHECK(e <= 5 * u * u, "df_mul err %Lg u^2", e / (u * u));
    }
    // Fused: the product's error (relative to |ab|) plus the sum's (relative
    // to the result), as an absolute bound.
    const long double ef = std::fabs(pair_value(ttg::df_fma(a, b, c)) - f);
    const long double bound = 5 * u * u * std::fabs(p) + 3 * u * u * (std::fabs(f) + std::fabs(p) * 5 * u * u);
    if (f != 0.0L)
      wf = std::fmax(wf, static_cast<double>(ef / (u * u * (std::fabs(p) + std::fabs(f)))));
    CHECK(ef <= bound * (1 + 1e-6L) + 1e-300L, "df_fma err %Lg bound %Lg", ef, bound);
  }
  std::printf("ops: worst df_add %.2f u^2 (bound 3), df_mul %.2f u^2 (bound 5), df_fma %.2f u^2 of "
              "|ab|+|ab+c|\n",
              wa, wm, wf);
}

static void check_recip_sqrt()
{
  std::mt19937_64 rng(11);
  std::uniform_real_distribution<double> u(0.5, 2.0);
  std::uniform_int_distribution<int> ek(-30, 30);
  double wr = 0.0, ws = 0.0;
  for (int it = 0; it < 200000; ++it)
  {
    const double v = std::ldexp(u(rng), ek(rng));
    const df64 b = ttg::df_split_pow2(v, 0);
    const long double bv = pair_value(b);
    const df64 r = ttg::df_recip(b);
    wr = std::fmax(wr, static_cast<double>(std::fabs(pair_value(r) * bv - 1.0L)));
    const df64 s = ttg::df_sqrt(b);
    const long double sv = pair_value(s);
    ws = std::fmax(ws, static_cast<double>(std::fabs(sv * sv / bv - 1.0L) / 2));
  }
  std::printf("recip: worst rel. err %.3g, sqrt %.3g (2^-45 = %.3g)\n", wr, ws, 0x1p-45);
  CHECK(wr <= 0x1p-45, "recip %g", wr);
  CHECK(ws <= 0x1p-45, "sqrt %g", ws);
  const df64 z = ttg::df_sqrt(df64{0.0f, 0.0f});
  CHECK(z.hi == 0.0f && z.lo == 0.0f, "sqrt(0)");
}

// Every product A(i, p) B(p, j) that can be non-zero must be formed by the
// tile containing (i, j), in a slab the tile visits, by the thread and block
// position whose rows/columns the live rule keeps; none outside the matrix.
static void check_gemm_live()
{
  std::mt19937 rng(3);
  long long products = 0;
  for (int trial = 0; trial < 60; ++trial)
  {
    const int M = 1 + static_cast<int>(rng() % 140), N = 1 + static_cast<int>(rng() % 140),
              K = 1 + static_cast<int>(rng() % 140);
    const int tri = static_cast<int>(rng() % 3);  // none, upper A, lower B
    for (int i0 = 0; i0 < M; i0 += 64)
      for (int j0 = 0; j0 < N; j0 += 64)
      {
        const int pstart = tri == 1 ? i0 : (tri == 2 ? j0 : 0);
        for (int ii = 0; ii < 64; ++ii)
          for (int jj = 0; jj < 64; ++jj)
          {
            const int i = i0 + ii, j = j0 + jj, ty = ii & 15, a = ii >> 4, tx = jj & 15,
                      b = jj >> 4;
            for (int p = 0; p < K; ++p)
            {
              const int p0 = (p / 16) * 16;
              const bool visited = p0 >= pstart;
              const int na = ttg::gemm_live(M - i0, ty, tri == 1, p0 - i0);
              const int nb = ttg::gemm_live(N - j0, tx, tri == 2, p0 - j0);
              const bool formed = visited && a < na && b < nb;
              const bool inside = i < M && j < N;
              const bool nonzero = inside && !(tri == 1 && p < i) && !(tri == 2 && p < j);
              if (nonzero)
              {
                ++products;
                CHECK(formed, "missed product M=%d N=%d K=%d tri=%d i=%d j=%d p=%d", M, N, K,
                      tri, i, j, p);
              }
              if (!inside)
                CHECK(!formed, "product outside M=%d N=%d i=%d j=%d", M, N, i, j);
            }
          }
      }
  }
  std::printf("gemm_live: %lld non-zero products checked\n", products);
}

int main()
{
  check_split();
  check_ops();
  check_recip_sqrt();
  check_gemm_live();
  if (g_fail)
  {
    std::printf("%d failures\n", g_fail);
    return 1;
  }
  std::printf("OK\n");
  return 0;
}
