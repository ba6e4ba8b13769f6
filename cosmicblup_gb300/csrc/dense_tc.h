// Tensor-core (3xTF32) dense block product of the FP32 PCG bulk.
#pragma once
#include "handle.h"

namespace cbx {
// K splits for an ng x ld block (balances work units over the SMs, at most 8).
int dense_tc_ksplit(int64_t ng, int64_t ld, int num_sms);
// The same split with its grid and the 32-element K steps per CTA.
int dense_tc_stream_k(int64_t ng, int64_t ld, int num_sms, int* grid, int* per);
// Tpart[ks][i][c] = sum over split ks of Qd[i][k] Vt[c][k]; S = 16 or 32.
void dense_tc(cbx_handle* h, const float* Qd, int64_t ng, int64_t ld, const float* Vt, int S, int ksplit,
              float* Tpart, const int* active, int ncols);
// The bf16 block product (dense_bf.cu): the same split over 64-element K steps,
// the bf16 copy of Qd - shift, and Tpart as dense_tc for the first ncols of the
// S gathered FP32 rows Vt (Vhl: 2 S ld bf16 scratch); returns the partial count.
int dense_bf_stream_k(int64_t ng, int64_t ld, int num_sms, int* grid, int* per);
void dense_bf_block(cbx_handle* h, const double* Qd64, int64_t ng, int64_t ld, double shift, uint16_t* Qbf);
int dense_bf(cbx_handle* h, const uint16_t* Qbf, int64_t ng, int64_t ld, const float* Vt, int S, uint16_t* Vhl,
             float* Tpart, const int* active, int ncols);
// FP64-accurate block product on the tensor cores by exact fixed-point digits
// (dense_fx.cu): Tout[i * os + c] = sum_k (qh + ql)[i][k] v[k][c] for c < ncols <= 32,
// v[k][c] = X[(p + gmap[k]) * xs + c] (k < ng), the block an ng x ld row-major pair of
// FP32 planes.  rowexp holds the row scales from fx_row_scales; bdig, cexp and part are
// scratch sized here.
void fx_row_scales(cbx_handle* h, const float* qh, int64_t ng, int64_t ld, int32_t* rowexp);
void fx_product(cbx_handle* h, const float* qh, const float* ql, const int32_t* rowexp, int64_t ng, int64_t ld,
                const double* X, int xs, int64_t p, const int32_t* gmap, int ncols, DevBuf<uint16_t>& bdig,
                DevBuf<int32_t>& cexp, DevBuf<double>& part, double* Tout, int os, const int* active);
}  // namespace cbx
