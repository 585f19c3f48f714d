// Batch kernels under the int64_grid policy (float and double queries, every tuner configuration).
#include "batch_kernels.cuh"

namespace agwn
{
const BatchPolicyOps kBatchP64 = {sizeof(RSeg<P64::C>), true, &BatchOpsFor<P64>::occupancy,
                                &BatchOpsFor<P64>::launch};
} // namespace agwn
