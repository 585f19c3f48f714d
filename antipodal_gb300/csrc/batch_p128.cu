// Batch kernels under the int128_grid policy (float and double queries, every tuner configuration).
#include "batch_kernels.cuh"

namespace agwn
{
const BatchPolicyOps kBatchP128 = {sizeof(RSeg<P128::C>), false, &BatchOpsFor<P128>::occupancy,
                                &BatchOpsFor<P128>::launch};
} // namespace agwn
