// Batch kernels under the exact_float policy (float and double queries, every tuner configuration).
#include "batch_kernels.cuh"

namespace agwn
{
const BatchPolicyOps kBatchPF = {sizeof(RSeg<PF::C>), false, &BatchOpsFor<PF>::occupancy,
                                &BatchOpsFor<PF>::launch};
} // namespace agwn
