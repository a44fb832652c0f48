// Split-precision tall products on the tensor cores (placeholder until the
// tcgen05 kernels land: reports the shape as unsupported).
#include "common.cuh"
#include "split.h"

namespace bcgs {

bool split_supported(i64, int, int) { return false; }
i64 split_workspace_bytes(i64, int, int, int) { return 0; }
int launch_gram_split(const double*, i64, i64, int, int, int, double*, int, char*, size_t, int,
                      cudaStream_t) {
    return (int)cudaErrorNotSupported;
}
int launch_update_split(double*, i64, i64, int, int, int, const double*, int, const double*, int,
                        char*, size_t, int, cudaStream_t) {
    return (int)cudaErrorNotSupported;
}

}  // namespace bcgs
