// lq_batch_mixed.cu -- batched-ensemble instantiations (D = 2, 3, 4), FP32 arithmetic on compensated (hi, lo) FP32 storage.
#include "batch_engine.cuh"

namespace lq {
const BatchOps *batch_ops_mixed(int dim) {
    switch (dim) {
    case 2: return BatchEngine<2, float, true>::table();
    case 3: return BatchEngine<3, float, true>::table();
    case 4: return BatchEngine<4, float, true>::table();
    default: return nullptr;
    }
}
} // namespace lq
