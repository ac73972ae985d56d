// Host check of the double-float routines (nfempy_gb300/csrc/df64.cuh)
// against long double: random operands over many binades, the largest
// relative error of each operation printed as "name max_rel".
#include <cmath>
#include <cstdio>
#include <random>

#include "../../nfempy_gb300/csrc/df64.cuh"

using nfem::dfloat;
static long double val(dfloat x) { return (long double)x.hi + (long double)x.lo; }

int main() {
  std::mt19937_64 g(20261204);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::uniform_int_distribution<int> ex(-40, 40);
  auto rnd = [&]() { return std::ldexp(u(g), ex(g)); };
  long double e_split = 0, e_pack = 0, e_add = 0, e_mul = 0, e_rec = 0, e_dot = 0, e_round = 0, e_i64 = 0;
  long double e_q64 = 0, e_prod = 0, e_scaled = 0;
  bool i32_exact = true;
  std::uniform_int_distribution<int> tb(1, 31), eo(-1080, 920);
  std::uniform_int_distribution<int64_t> iq(-(int64_t(1) << 62), int64_t(1) << 62);
  std::uniform_int_distribution<int> sh(0, 120);
  for (int it = 0; it < 200000; ++it) {
    double a = rnd(), b = rnd(), c = rnd();
    if (a == 0 || b == 0 || c == 0) continue;
    dfloat A = nfem::df_from_double(a), B = nfem::df_from_double(b), C = nfem::df_from_double(c);
    e_split = std::fmax(e_split, std::fabs((val(A) - a) / a));
    // round trip of a normalised pair through FP64
    dfloat An = nfem::quick_two_sum(A.hi, A.lo);
    double back = nfem::df_to_double(An);
    e_round = std::fmax(e_round, std::fabs(((long double)back - val(An)) / val(An)));
    long double ra = a, rb = b;
    dfloat s = nfem::df_add(A, B);
    e_add = std::fmax(e_add, std::fabs(val(s) - (ra + rb)) / (std::fabs(ra) + std::fabs(rb)));
    dfloat p = nfem::df_mul(A, B);
    e_mul = std::fmax(e_mul, std::fabs((val(p) - ra * rb) / (ra * rb)));
    dfloat r = nfem::df_recip(A);
    e_rec = std::fmax(e_rec, std::fabs((val(r) - 1.0L / ra) * ra));
    dfloat x3[3] = {A, B, C}, y3[3] = {C, A, B};
    float sg[3] = {1.f, -1.f, 1.f};
    dfloat d = nfem::df_dot<3>(x3, y3, sg);
    long double td = (long double)a * c - (long double)b * a + (long double)c * b;
    long double scale = std::fabs((long double)a * c) + std::fabs((long double)b * a) + std::fabs((long double)c * b);
    e_dot = std::fmax(e_dot, std::fabs(val(d) - td) / scale);
    // fixed-point integers over all magnitudes (shifted right by a random amount of bits)
    int64_t qi = iq(g) >> (it % 62);
    int shift = sh(g);
    if (qi != 0) {
      dfloat Q = nfem::df_from_i64(qi, shift);
      long double want = std::ldexp((long double)qi, -shift);
      e_i64 = std::fmax(e_i64, std::fabs((val(Q) - want) / want));
    }
    // the lattice records: V 2^68 as a 64-bit integer for V in (1/120, 1/30],
    // and t vq 2^e as FP64 for integers t of any size and sign
    {
      dfloat V = nfem::df_recip(nfem::df_mul_f(nfem::df_from_double(1.0 + std::fabs(u(g)) * 3.0), 30.f));
      V = nfem::quick_two_sum(V.hi, V.lo);
      uint64_t vq = nfem::df_to_u64_scaled(V, 68);
      long double want = std::ldexp(val(V), 68);
      e_q64 = std::fmax(e_q64, std::fabs(((long double)vq - want) / want));
      const uint64_t vqn = vq << __builtin_clzll(vq);  // normalised to [2^63, 2^64)
      int32_t t = static_cast<int32_t>(g() >> (64 - tb(g)));
      if (g() & 1) t = -t;
      int e = eo(g);
      double r = nfem::df_i32_times_q63(t, vqn, e);
      long double exact = std::ldexp((long double)t * (long double)vqn, e);
      if (t == 0 && r != 0.0) e_prod = 1.0L;
      if (t != 0) e_prod = std::fmax(e_prod, std::fabs(((long double)r - exact) / exact));
      double rs = nfem::df_to_double_scaled(V, e);
      long double es = std::ldexp(val(V), e);
      if (std::fabs(es) > 1e-300L && std::fabs(es) < 1e300L)
        e_scaled = std::fmax(e_scaled, std::fabs(((long double)rs - es) / es));
    }
    // 32-bit integers to FP64 by bits: exact
    {
      const int32_t t = static_cast<int32_t>(g()) >> (it % 31);
      if (nfem::df_i32_to_double(t) != static_cast<double>(t)) i32_exact = false;
    }
    // packing of a normalised pair whose hi is a power of two and lo points below it
    dfloat q = nfem::quick_two_sum(std::ldexp(1.0f, ex(g)), -std::ldexp((float)std::fabs(u(g)), -30 + ex(g)));
    double qd = nfem::df_to_double(q);
    e_pack = std::fmax(e_pack, std::fabs(((long double)qd - val(q)) / val(q)));
  }
  std::printf("split %.9Le\nround %.9Le\npack %.9Le\nadd %.9Le\nmul %.9Le\nrecip %.9Le\ndot %.9Le\ni64 %.9Le\n",
              e_split, e_round, e_pack, e_add, e_mul, e_rec, e_dot, e_i64);
  std::printf("q64 %.9Le\nprod %.9Le\nscaled %.9Le\n", e_q64, e_prod, e_scaled);
  std::printf("i32 %d\n", (i32_exact && nfem::df_i32_to_double(INT32_MIN) == -2147483648.0 &&
                           nfem::df_i32_to_double(0) == 0.0 && nfem::df_i32_to_double(-1) == -1.0) ? 0 : 1);
  return 0;
}
