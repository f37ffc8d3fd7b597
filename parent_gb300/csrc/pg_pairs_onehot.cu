// Pair kernel, tensor-core one-hot form (placeholder until the tcgen05
// kernel lands) and the form autotuner.
#include "../../include/parent_gb300.h"
#include "pg_internal.h"

namespace pg {

bool pairs_onehot_supported(const SysGeom &) { return false; }
size_t pairs_onehot_scratch_bytes(const SysGeom &) { return 256; }
cudaError_t launch_pairs_onehot(const SysGeom &, const uint8_t *, const DofArrays &, const double *,
                                PairOut, int *, cudaStream_t, void *, size_t, int *launches) {
    *launches = 0;
    return cudaErrorNotSupported;
}
int autotune_form(const SysGeom &) { return PG_FORM_HIST; }

}  // namespace pg
