/* Checks the division-free v / pi of the search's epilogue (k_finish_outputs:
 * q0 = RN(v * RN(1/pi)), r = fma(-q0, pi, v), q = fma(r, RN(1/pi), q0))
 * against IEEE division on the host: every operation is a single correctly
 * rounded IEEE operation, so the host and the GPU give the same bits.
 * Inputs: lattice sums j * 0.25 deg as the search forms them (chains of
 * +-0.5 deg steps from 0, then +-0.25 deg), each with its 64 nearest
 * neighbours, sector sums of up to 50 such values, and log-uniform random
 * doubles over [2^-12, 2^12]. Prints the number of values and mismatches. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#define PI_RN 3.14159265358979323846 /* RN(pi), the value of M_PI */

static double div_pi_rn(double v) {
  const double y = 1.0 / PI_RN;
  const double q0 = v * y;
  const double r = fma(-q0, PI_RN, v);
  return fma(r, y, q0);
}

static uint64_t state = 0x9e3779b97f4a7c15ull;
static uint64_t next_u64(void) { /* xorshift64* */
  state ^= state >> 12;
  state ^= state << 25;
  state ^= state >> 27;
  return state * 0x2545f4914f6cdd1dull;
}
static double uniform(void) { return (double)(next_u64() >> 11) * (1.0 / 9007199254740992.0); }

static long long checked = 0, bad = 0;
static void check(double v) {
  checked++;
  if (div_pi_rn(v) != v / PI_RN) {
    if (bad < 10) printf("mismatch v=%a div=%a fma=%a\n", v, v / PI_RN, div_pi_rn(v));
    bad++;
  }
}

int main(int argc, char** argv) {
  const long long n_random = argc > 1 ? atoll(argv[1]) : 4000000;
  const double ha = 0.25 / 180.0 * PI_RN;
  /* Elevation walks: random +-2ha steps from 0 (as the chained search carries
   * them across azimuths), each visited value closed with +-ha. */
  for (int walk = 0; walk < 2000; walk++) {
    double elev = 0.0;
    for (int step = 0; step < 400; step++) {
      elev += (next_u64() & 1) ? (2.0 * ha) : -(2.0 * ha);
      if (elev < -1.4) elev += 2.0 * ha * 10;
      for (int sgn = -1; sgn <= 1; sgn += 2) {
        double h = elev + sgn * ha;
        if (h <= 0.0) continue;
        check(h);
        double up = h, dn = h;
        for (int k = 0; k < 32; k++) {
          up = nextafter(up, INFINITY);
          dn = nextafter(dn, 0.0);
          check(up);
          check(dn);
        }
      }
    }
  }
  /* Sector sums of refine_factor values. */
  for (int t = 0; t < 200000; t++) {
    const int refine = 2 + (int)(next_u64() % 49);
    double sum = 0.0;
    for (int k = 0; k < refine; k++) sum += (double)(1 + 2 * (int)(next_u64() % 360)) * ha;
    check(sum);
  }
  for (long long t = 0; t < n_random; t++) check(ldexp(1.0 + uniform(), -12 + (int)(next_u64() % 24)));
  printf("checked %lld mismatches %lld\n", checked, bad);
  return bad != 0;
}
