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
// Same contracts as launch_gram_fp64 / launch_update_fp64.
int launch_gram_split(const double* X, i64 ld, i64 m, int na, int b0, int nb, double* out, int ldo,
                      char* ws, size_t ws_bytes, int num_sms, cudaStream_t st);
int launch_update_split(double* X, i64 ld, i64 m, int K, int c0, int nc, const double* S, int lds,
                        const double* T, int ldt, char* ws, size_t ws_bytes, int num_sms,
                        cudaStream_t st);

}  // namespace bcgs
