// lq_mixed.cu -- mixed-precision instantiations (D = 2, 3, 4): FP32 arithmetic on compensated
// FP32 pairs (hi + lo) for the stored links and E-field; every reduction accumulates in FP64.
#include "engine.cuh"

namespace lq {
const Ops *ops_mixed(int dim) {
    switch (dim) {
    case 2: return Engine<2, float, true>::table();
    case 3: return Engine<3, float, true>::table();
    case 4: return Engine<4, float, true>::table();
    default: return nullptr;
    }
}
} // namespace lq
