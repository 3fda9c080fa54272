// lq_f32.cu -- FP32 instantiations (D = 2, 3, 4) with plain FP32 storage of links and E-field;
// every reduction accumulates in FP64.
#include "engine.cuh"

namespace lq {
const Ops *ops_f32(int dim) {
    switch (dim) {
    case 2: return Engine<2, float, false>::table();
    case 3: return Engine<3, float, false>::table();
    case 4: return Engine<4, float, false>::table();
    default: return nullptr;
    }
}
} // namespace lq
