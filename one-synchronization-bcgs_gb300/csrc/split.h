// Split-precision (tensor-core) forms of the tall products. Declared here so the
// C-ABI layer can dispatch on the precision mode.
#pragma once

#include <cuda_runtime.h>

namespace bcgs {

using i64 = long long;

// Whether the split-precision path handles this shape.
bool split_supported(i64 m, int n, int s);
// Workspace bytes the split path needs for (m, n, s).
i64 split_workspace_bytes(i64 m, int n, int s, int num_sms);
// Start a split-precision run on X (m x n, ld): lays out the digit stores in the
// workspace, encodes the TMA maps and marks every column's digits stale.
// kd: digit planes per operand, 7 (56-bit) or 6 (48-bit).
int split_begin(double* X, i64 ld, i64 m, int n, int s, int kd, char* ws, size_t ws_bytes, int num_sms,
                cudaStream_t st);
// Bring the digit planes of columns [0, c_end) up to date (slices stale columns).
int split_prepare(int c_end, cudaStream_t st);
// Digit planes per operand of the current run.
int split_digits();
// Columns [c0, c0+nc) of X were rewritten outside the split kernels.
void split_mark_stale(int c0, int nc);
// The digit planes of all n columns of X (m x n, ld) in the store's layout
// ([plane][64-row chunk][column][64 rows], ceil(m / 64) chunks), each column's
// scale exponent into cexp[n]; cmax: n words of scratch. kd: 6 or 7.
int split_slice_columns(const double* X, i64 ld, i64 m, int n, int kd, unsigned short* digits, int* cexp,
                        unsigned long long* cmax, cudaStream_t st);
// Reads (and waits for) the split kernels' error word: 0, or the code of a wait
// that ran out.
int split_error_word(int* out, cudaStream_t st);
// Device address of the error word of the current run (valid after split_begin).
int* split_error_ptr();
// Selects the plan (digit stores, maps, freshness) the calls above use: 0 .. 7.
void split_select_slot(int slot);
// Forget which workspaces were zeroed (call after freeing them).
void split_forget_workspaces();
// Last nonzero error word seen: the code of the bounded wait that ran out (for the
// A-ring waits, code + 100 * ring slot).
int split_last_error();
// Same contracts as launch_gram_fp64 / launch_update_fp64 (the update requires
// c0 == K and nc <= 64; output columns are written in groups of 32).
int launch_gram_split(const double* X, i64 ld, i64 m, int na, int b0, int nb, double* out, int ldo,
                      char* ws, size_t ws_bytes, int num_sms, cudaStream_t st);
int launch_update_split(double* X, i64 ld, i64 m, int K, int c0, int nc, const double* S, int lds,
                        const double* T, int ldt, char* ws, size_t ws_bytes, int num_sms,
                        cudaStream_t st);

// Fused update of the lagged one-sync variants (s, nz <= 64), in one product over
// X[:, 0:K+s+nz]: X[:, K:K+s] = (U_k - Q Y) Ty^{-1} (Y = G[0:K, 0:s]) and
// X[:, K+s:K+s+nz] = (X_{k+1} - [Q Q_k] S') Ts^{-1} (S' = Sp, K+s rows; Ts may be null).
int launch_fused_update_split(double* X, i64 ld, i64 m, int K, int s, int nz, const double* G, int ldg,
                              const double* Ty, const double* Sp, int ldsp, const double* Ts, int num_sms,
                              cudaStream_t st);

// Staged split-precision batches (BCGSI+P-1S, s <= 16): one launch per stage for
// all matrices of a wave, each wave one captured graph (split_bf16.cu).
struct SplitStaged;
bool split_staged_supported(int variant, int count, const int* s);
// kd: 7 or 6 digit planes; dstatus: 8 ints per matrix on the device (status words,
// split error word); budget: bytes of device memory for a wave (< 0: from the free
// memory). Returns 0, 2 (invalid shapes) or 3.
int split_staged_create(int count, const int* m, const int* n, const int* s, double* const* dX,
                        const long long* ldX, double* const* dR, const int* ldR, int kd, int* dstatus,
                        long long budget, cudaStream_t st, SplitStaged** out);
int split_staged_run(SplitStaged* plan, cudaStream_t st);
void split_staged_destroy(SplitStaged* plan);
void split_staged_info(const SplitStaged* plan, long long* kernels, long long* bytes, int* nodes, int* waves);
// The same planning without a GPU: waves, kernel launches per run and the wave
// buffer's bytes for a given budget.
int split_staged_dry_run(int count, const int* m, const int* n, const int* s, long long budget, int* waves,
                         long long* kernels, long long* bytes);

}  // namespace bcgs
