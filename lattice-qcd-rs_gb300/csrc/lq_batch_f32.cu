// lq_batch_f32.cu -- batched-ensemble instantiations (D = 2, 3, 4), plain FP32 storage and arithmetic.
#include "batch_engine.cuh"

namespace lq {
const BatchOps *batch_ops_f32(int dim) {
    switch (dim) {
    case 2: return BatchEngine<2, float, false>::table();
    case 3: return BatchEngine<3, float, false>::table();
    case 4: return BatchEngine<4, float, false>::table();
    default: return nullptr;
    }
}
} // namespace lq
