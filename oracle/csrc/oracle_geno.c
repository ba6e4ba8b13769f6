/* Oracle (test infrastructure): restatement of PlinkReader::multiply_Zt_v, reference
 * src/core/plink_reader.cpp:341-392, for SNPs [j0, j1).  Per SNP, in sample order:
 * for every observed code (01 = missing is skipped) sum_xv += (double)(float)x * v_i
 * and sum_v_obs += v_i, with x = 2, 1, 0 for codes 00, 10, 11; then
 * y_j = (sum_xv - mean_j sum_v_obs) inv_std_j, or 0 when inv_std_j == 0.
 * The reference parallelises over SNPs with OpenMP; callers run disjoint SNP ranges
 * on several threads. */
#include <stdint.h>

void oracle_multiply_zt_v(const uint8_t* payload, int64_t n, int64_t bps, const double* mean,
                          const double* inv_std, const double* v, double* y, int64_t j0, int64_t j1) {
  static const float lut[4] = {2.0f, 0.0f, 1.0f, 0.0f};
  for (int64_t j = j0; j < j1; ++j) {
    const double is = inv_std[j];
    if (is == 0.0) {
      y[j] = 0.0;
      continue;
    }
    const uint8_t* col = payload + j * bps;
    double sum_xv = 0.0, sum_v_obs = 0.0;
    for (int64_t b = 0; b < bps; ++b) {
      const uint8_t byte = col[b];
      for (int k = 0; k < 4; ++k) {
        const int64_t idx = 4 * b + k;
        if (idx >= n) break;
        const unsigned code = (byte >> (2 * k)) & 3u;
        if (code != 1u) {
          const double vi = v[idx];
          sum_xv += (double)lut[code] * vi;
          sum_v_obs += vi;
        }
      }
    }
    y[j] = (sum_xv - mean[j] * sum_v_obs) * is;
  }
}
