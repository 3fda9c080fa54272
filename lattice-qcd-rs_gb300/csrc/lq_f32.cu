// lq_f32.cu -- FP32 instantiations (D = 2, 3, 4): the bulk of the mixed-precision form
// (links, E-field and force in FP32; every reduction accumulates in FP64).
#include "engine.cuh"

namespace lq {
const Ops *ops_f32(int dim) {
    switch (dim) {
    case 2: return Engine<2, float>::table();
    case 3: return Engine<3, float>::table();
    case 4: return Engine<4, float>::table();
    default: return nullptr;
    }
}
} // namespace lq
