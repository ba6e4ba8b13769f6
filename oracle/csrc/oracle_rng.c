/* Oracle (test infrastructure): restatement of the probe generator of the
 * reference, src/core/rng.h:19-53 -- std::mt19937_64 seeded with `seed`, and
 * fill_rademacher = std::uniform_int_distribution<int>(0, 1) mapping 0 -> -1.
 * With a 64-bit engine libstdc++ draws that distribution by Lemire's
 * multiply-shift on 128 bits: value = (x * 2) >> 64, i.e. the top bit of x.
 * mt19937_64 is the published Matsumoto-Nishimura 64-bit Mersenne Twister. */
#include <stdint.h>

#define NN 312
#define MM 156
#define MATRIX_A 0xB5026F5AA96619E9ULL
#define UM 0xFFFFFFFF80000000ULL
#define LM 0x7FFFFFFFULL

typedef struct { uint64_t mt[NN]; int mti; } mt64_t;

static void mt64_seed(mt64_t* s, uint64_t seed) {
  s->mt[0] = seed;
  for (int i = 1; i < NN; ++i)
    s->mt[i] = 6364136223846793005ULL * (s->mt[i - 1] ^ (s->mt[i - 1] >> 62)) + (uint64_t)i;
  s->mti = NN;
}

static uint64_t mt64_next(mt64_t* s) {
  static const uint64_t mag01[2] = {0ULL, MATRIX_A};
  if (s->mti >= NN) {
    int i;
    uint64_t x;
    for (i = 0; i < NN - MM; ++i) {
      x = (s->mt[i] & UM) | (s->mt[i + 1] & LM);
      s->mt[i] = s->mt[i + MM] ^ (x >> 1) ^ mag01[(int)(x & 1ULL)];
    }
    for (; i < NN - 1; ++i) {
      x = (s->mt[i] & UM) | (s->mt[i + 1] & LM);
      s->mt[i] = s->mt[i + (MM - NN)] ^ (x >> 1) ^ mag01[(int)(x & 1ULL)];
    }
    x = (s->mt[NN - 1] & UM) | (s->mt[0] & LM);
    s->mt[NN - 1] = s->mt[MM - 1] ^ (x >> 1) ^ mag01[(int)(x & 1ULL)];
    s->mti = 0;
  }
  uint64_t x = s->mt[s->mti++];
  x ^= (x >> 29) & 0x5555555555555555ULL;
  x ^= (x << 17) & 0x71D67FFFEDA60000ULL;
  x ^= (x << 37) & 0xFFF7EEE000000000ULL;
  x ^= (x >> 43);
  return x;
}

/* `count` probes of length n, drawn consecutively from one engine seeded with `seed`. */
void oracle_rademacher(uint64_t seed, int64_t n, int64_t count, double* out) {
  mt64_t s;
  mt64_seed(&s, seed);
  for (int64_t i = 0; i < n * count; ++i) out[i] = (mt64_next(&s) >> 63) ? 1.0 : -1.0;
}

/* raw engine output, for checking against published mt19937_64 values */
void oracle_mt64_raw(uint64_t seed, int64_t count, uint64_t* out) {
  mt64_t s;
  mt64_seed(&s, seed);
  for (int64_t i = 0; i < count; ++i) out[i] = mt64_next(&s);
}
