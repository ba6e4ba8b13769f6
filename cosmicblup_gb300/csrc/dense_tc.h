// Tensor-core (3xTF32) dense block product of the FP32 PCG bulk.
#pragma once
#include "handle.h"

namespace cbx {
// K splits for an ng x ld block (balances work units over the SMs, at most 8).
int dense_tc_ksplit(int64_t ng, int64_t ld, int num_sms);
// Tpart[ks][i][c] = sum over split ks of Qd[i][k] Vt[c][k]; S = 16 or 32.
void dense_tc(cbx_handle* h, const float* Qd, int64_t ng, int64_t ld, const float* Vt, int S, int ksplit,
              float* Tpart, const int* active, int ncols);
}  // namespace cbx
