// Sort-then-deposit CIC scatter (SC_DEPOSIT_SORTED / SC_DEPOSIT_DETERMINISTIC).
#include "sc_internal.cuh"

namespace sc {

int deposit_sorted_launch(sc_mesh* m, const void* x, const void* y, const void* z, const void* q, int64_t n,
                          int dtype, int mode, cudaStream_t s) {
    (void)m, (void)x, (void)y, (void)z, (void)q, (void)n, (void)dtype, (void)mode, (void)s;
    return fail(SC_ERR_UNSUPPORTED, "sorted deposit is not available in this build");
}

}  // namespace sc
