// MIST without any device allocation, for callers that cannot call cudaMalloc.
//
// Some host programs that would embed this library own the whole device
// memory budget themselves: an MD engine or an analysis service that
// pre-allocates one pool at start-up and forbids further allocations, or a
// caller that cannot afford the implicit device-wide synchronisation that
// cudaMalloc/cudaFree may perform while its other streams are busy. Such a
// caller hands over its own device buffers for the MI matrix and the edge list
// and needs the library to allocate nothing.
//
// The only memory the MIST kernel needs beyond its inputs and outputs is its
// per-DOF scratch (best key, best partner, insertion position: 16 bytes per
// DOF). Here it lives in a file-scope __device__ array sized for
// PG_NOALLOC_MAX_DOFS DOFs, which every GPU that loads the library keeps
// until the process exits.
#include "../../include/parent_gb300.h"
#include "pg_internal.h"

namespace pg {
cudaError_t launch_mist_impl(int D, int nb, int na, const double *mi, void *scratch,
                             double *edge_mi, int *edge_from, int *edge_to, cudaStream_t st);
size_t mist_scratch_bytes(int D);
void set_global_error(const char *msg);
}  // namespace pg

namespace {

// key[D] (double) | from[D] (int) | pos[D] (int), plus the 256 B pad the
// allocating path also reserves (mist_scratch_bytes).
constexpr size_t kScratchBytes = (size_t)PG_NOALLOC_MAX_DOFS * 16 + 256;
__device__ __align__(256) unsigned char g_mist_scratch[kScratchBytes];

// Device address of g_mist_scratch on the current device. In host code the
// array's name is only a host-side stand-in, so the address is looked up
// with the device current. The lookup is repeated on every call (it is cheap
// and enqueues nothing): a cached address would dangle after the host program
// resets the device, which reloads the module.
int scratch_for_current_device(void **out) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_mist_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();  // leave no error of this lookup behind
        pg::set_global_error(e != cudaSuccess ? cudaGetErrorString(e) : "pg_mist_noalloc: null scratch address");
        return PG_ERR_CUDA;
    }
    *out = p;
    return PG_OK;
}

}  // namespace

extern "C" PG_API int pg_mist_noalloc(int n_dihedrals, const double *mi, double *edge_mi,
                                      int *edge_from, int *edge_to, void *stream) {
    if (n_dihedrals < 0) {
        pg::set_global_error("pg_mist_noalloc: n_dihedrals < 0");
        return PG_ERR_ARG;
    }
    const long long D = 3LL * n_dihedrals + 3;
    if (D > PG_NOALLOC_MAX_DOFS) {
        pg::set_global_error("pg_mist_noalloc: 3*n_dihedrals+3 DOFs exceed PG_NOALLOC_MAX_DOFS (16384); "
                             "use pg_mist for larger systems");
        return PG_ERR_UNSUPPORTED;
    }
    if (!mi || !edge_mi || !edge_from || !edge_to) {
        pg::set_global_error("pg_mist_noalloc: null device pointer");
        return PG_ERR_ARG;
    }
    if (pg::mist_scratch_bytes((int)D) > kScratchBytes) {
        pg::set_global_error("pg_mist_noalloc: scratch layout larger than the static array");
        return PG_ERR_UNSUPPORTED;
    }
    // an error left by the host program's own earlier CUDA calls on this
    // thread is not this call's
    cudaGetLastError();
    void *scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc != PG_OK) return rc;
    // Only the one-CTA kernel on more DOFs than its shared memory holds
    // (above 12,800 DOFs, with the cluster kernel switched off by
    // PG_MIST_CLUSTER=0) keeps its per-DOF arrays in this static array; the
    // other kernels keep them in shared memory. That kernel initialises every
    // key/from entry it reads and writes each insertion position before
    // reading it, so leftover contents of an earlier call need no clearing.
    const int nb = n_dihedrals + 2, na = n_dihedrals + 1;
    cudaError_t e = pg::launch_mist_impl((int)D, nb, na, mi, scratch, edge_mi, edge_from, edge_to,
                                         (cudaStream_t)stream);
    if (e != cudaSuccess) {
        pg::set_global_error(cudaGetErrorString(e));
        return PG_ERR_CUDA;
    }
    return PG_OK;
}
