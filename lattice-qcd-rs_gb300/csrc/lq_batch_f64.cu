// lq_batch_f64.cu -- batched-ensemble instantiations (D = 2, 3, 4), FP64 arithmetic and storage.
#include "batch_engine.cuh"

namespace lq {
const BatchOps *batch_ops_f64(int dim) {
    switch (dim) {
    case 2: return BatchEngine<2, double, false>::table();
    case 3: return BatchEngine<3, double, false>::table();
    case 4: return BatchEngine<4, double, false>::table();
    default: return nullptr;
    }
}
} // namespace lq
