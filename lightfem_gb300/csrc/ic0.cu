// Incomplete Cholesky IC(0) on the GPU (placeholder until the level-scheduled
// factorisation and sweeps land).
#include "common.cuh"
#include "kernels.hpp"

namespace lfgpu {

void ensure_ic0(Context&, bool) { throw Error{LFGPU_ERR_UNSUPPORTED, "ic0 is not built yet"}; }

PcgResult run_pcg_ic0(Context&, const SolveSetup&, float*, double*) {
    throw Error{LFGPU_ERR_UNSUPPORTED, "ic0 is not built yet"};
}

}  // namespace lfgpu
