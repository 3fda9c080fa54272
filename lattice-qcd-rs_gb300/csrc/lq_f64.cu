// lq_f64.cu -- FP64 instantiations (D = 2, 3, 4): the parity form of the library.
#include "engine.cuh"

namespace lq {
const Ops *ops_f64(int dim) {
    switch (dim) {
    case 2: return Engine<2, double, false>::table();
    case 3: return Engine<3, double, false>::table();
    case 4: return Engine<4, double, false>::table();
    default: return nullptr;
    }
}
} // namespace lq
