// Host check of exadem_gb300/csrc/emu64.cuh: emu_dmul, emu_mul2, emu_mulhalf and
// emu_dadd_nb / emu_dsub_nb against the host's IEEE binary64 multiply and
// addition, bit for bit.
// Usage: emu64_check <n_cases> <seed>; prints "cases <n> mismatches <m>".
// Built by tests/test_emu64.py with g++ -O2 -ffp-contract=off.
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "emu64.cuh"

static uint64_t sm_state;
static uint64_t next64() {
  uint64_t z = (sm_state += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

static uint64_t bits(double x) { return dem::emu_bits(x); }

// operand classes: full random significand over a wide exponent band, short
// significands (exact products and ties), boundary exponents, and specials
static double draw() {
  const uint64_t r = next64();
  const uint64_t sign = (r & 1) << 63;
  const int cls = (int)((r >> 1) % 16);
  uint64_t frac = next64() & 0xfffffffffffffull;
  uint64_t e;
  if (cls < 7) {
    e = 1023 - 60 + (next64() % 121);  // typical magnitudes 2^-60..2^60
  } else if (cls < 10) {
    const int keep = (int)(next64() % 12);  // short significand: ties and exact products
    frac &= ~((1ull << (52 - keep)) - 1);
    e = 1023 - 30 + (next64() % 61);
  } else if (cls < 12) {
    e = 1 + (next64() % 2046);  // whole normal range: overflow / underflow of the product
  } else if (cls == 12) {
    e = (next64() & 1) ? 1 + (next64() % 40) : 2046 - (next64() % 40);
  } else if (cls == 13) {
    e = 0;  // zero or subnormal
    if (next64() & 1) frac = 0;
  } else if (cls == 14) {
    e = 2047;  // infinity or NaN
    if (next64() & 1) frac = 0;
  } else {
    frac = (next64() & 1) ? 0xfffffffffffffull : 0;  // all-ones / power of two significands
    e = 1023 - 8 + (next64() % 17);
  }
  double x;
  const uint64_t u = sign | (e << 52) | frac;
  memcpy(&x, &u, 8);
  return x;
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 1000000;
  sm_state = argc > 2 ? strtoull(argv[2], 0, 10) : 1;
  long bad = 0, flagged = 0;
  for (long i = 0; i < n; i++) {
    const double a = draw(), b = draw();
    const double ref = a * b, got = dem::emu_dmul(a, b);
    const bool nan_both = ref != ref && got != got;
    if (bits(ref) != bits(got) && !nan_both) {
      if (bad < 8)
        printf("mul %016llx * %016llx: want %016llx got %016llx\n", (unsigned long long)bits(a),
               (unsigned long long)bits(b), (unsigned long long)bits(ref), (unsigned long long)bits(got));
      bad++;
    }
    bool fl = false;
    const double gnb = dem::emu_dmul_nb(a, b, fl);
    if (!fl && bits(ref) != bits(gnb)) {
      if (bad < 8) printf("mul_nb %016llx * %016llx\n", (unsigned long long)bits(a), (unsigned long long)bits(b));
      bad++;
    }
    flagged += fl ? 1 : 0;
    const double sref[3] = {a * 2.0, a * 0.5, a * -0.5};
    bool f2 = false, fh = false, fn = false;
    const double snb[3] = {dem::emu_mul2_nb(a, f2), dem::emu_mulhalf_nb(a, fh), dem::emu_mulnhalf_nb(a, fn)};
    const bool sfl[3] = {f2, fh, fn};
    for (int q = 0; q < 3; q++)
      if (!sfl[q] && bits(sref[q]) != bits(snb[q])) {
        if (bad < 8) printf("scale_nb %d %016llx\n", q, (unsigned long long)bits(a));
        bad++;
      }
    const double r2 = a * 2.0, g2 = dem::emu_mul2(a);
    const double rh = a * 0.5, gh = dem::emu_mulhalf(a);
    const double rn = a * -0.5, gn = dem::emu_mulnhalf(a);
    if ((bits(r2) != bits(g2) && !(r2 != r2 && g2 != g2)) || (bits(rh) != bits(gh) && !(rh != rh && gh != gh)) ||
        (bits(rn) != bits(gn) && !(rn != rn && gn != gn))) {
      if (bad < 8) printf("scale %016llx\n", (unsigned long long)bits(a));
      bad++;
    }
  }
  // integer-pipe comparisons against the host's FP64 comparisons
  for (long i = 0; i < n / 4; i++) {
    const double a = draw(), b = draw();
    const double na = a * a, nb = b * b;  // +0, positive, inf or NaN
    const bool ok = dem::emu_gt0(a) == (a > 0) && dem::emu_lt0(a) == (a < 0) && dem::emu_ge0(a) == (a >= 0) &&
                    dem::emu_le0(a) == (a <= 0) && dem::emu_lt(a, b) == (a < b) && dem::emu_le(a, b) == (a <= b) &&
                    dem::emu_gt_nonneg(na, nb) == (na > nb) && dem::emu_ge_nonneg(na, nb) == (na >= nb) &&
                    dem::emu_lt(a, a) == (a < a) && dem::emu_le(a, -a) == (a <= -a);
    if (!ok) {
      if (bad < 8) printf("cmp %016llx %016llx\n", (unsigned long long)bits(a), (unsigned long long)bits(b));
      bad++;
    }
  }
  // zero addends
  for (long i = 0; i < n / 4; i++) {
    const double a = draw();
    const double z = (next64() & 1) ? -0.0 : 0.0;
    bool ok = false;
    const double got = dem::emu_add_zero(a, dem::emu_sign(z), ok);
    const double ref = a + z;
    if (ok && bits(got) != bits(ref)) {
      if (bad < 8) printf("addz %016llx %016llx\n", (unsigned long long)bits(a), (unsigned long long)bits(z));
      bad++;
    }
    if (!ok && a == a) bad++;  // only NaN may leave the fast path
  }
  // sums: independent operands, and pairs built for the cases addition branches
  // on (cancellation, exponent gaps 0..70, short significands for ties,
  // neighbours of -a, zeros)
  for (long i = 0; i < n; i++) {
    double a = draw(), b;
    const int cls = (int)(next64() % 6);
    if (cls == 0) {
      b = draw();
    } else if (cls == 1) {
      b = -a;
    } else if (cls == 2) {
      const uint64_t gap = next64() % 71, ua = bits(a);
      const uint64_t e = (ua >> 52) & 0x7ff;
      const uint64_t eb = e > gap ? e - gap : 1;
      uint64_t u = ((next64() & 1) << 63) | (eb << 52) | (next64() & 0xfffffffffffffull);
      memcpy(&b, &u, 8);
    } else if (cls == 3) {
      uint64_t u = bits(-a) + (next64() % 9) - 4;
      memcpy(&b, &u, 8);
    } else if (cls == 4) {
      const int keep = (int)(next64() % 10);
      uint64_t u = bits(draw()) & ~((1ull << (52 - keep)) - 1);
      memcpy(&b, &u, 8);
      uint64_t v = bits(a) & ~((1ull << 40) - 1);
      memcpy(&a, &v, 8);
    } else {
      b = (next64() & 1) ? 0.0 : -0.0;
    }
    bool fa = false, fs = false;
    const double ga = dem::emu_dadd_nb(a, b, fa), gs = dem::emu_dsub_nb(a, b, fs);
    const double ra = a + b, rs = a - b;
    if ((!fa && bits(ga) != bits(ra)) || (!fs && bits(gs) != bits(rs))) {
      if (bad < 8) printf("add %016llx + %016llx\n", (unsigned long long)bits(a), (unsigned long long)bits(b));
      bad++;
    }
    flagged += fa ? 1 : 0;
  }
  printf("flagged %ld (branch-free form: recomputed by the caller)\n", flagged);
  printf("cases %ld mismatches %ld\n", n, bad);
  return bad ? 1 : 0;
}
