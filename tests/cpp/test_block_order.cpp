// The launch order of the per-site stencil kernels is a permutation of their blocks: every block of
// 128 sites runs exactly once, for the lattice shapes where strips apply and where they do not.
#include <cstdio>
#include <vector>

#include "block_order.hpp"

int main() {
    const unsigned shapes[][2] = {{4, 8},  {4, 16}, {4, 24}, {4, 32}, {4, 40}, {4, 48}, {4, 64}, {4, 96},
                                  {3, 16}, {3, 64}, {3, 128}, {3, 256}, {3, 512}, {2, 512}, {2, 2048}};
    int bad = 0, strips = 0;
    for (const auto &sh : shapes) {
        const int D = (int)sh[0];
        const unsigned L = sh[1];
        unsigned long long V = 1;
        for (int i = 0; i < D; ++i) V *= L;
        const unsigned blocks = (unsigned)((V + 127) / 128);
        const lq::BlockOrder o = lq::make_block_order(D, L, 128, 32768);
        strips += o.on;
        if (o.on && (unsigned long long)o.nb * 128 * o.L * o.L != V) ++bad;
        std::vector<int> seen(blocks, 0);
        for (unsigned b = 0; b < blocks; ++b) {
            const unsigned s = lq::block_at(o, b);
            if (s >= blocks) { ++bad; continue; }
            ++seen[s];
        }
        for (unsigned s = 0; s < blocks; ++s) bad += seen[s] != 1;
        std::printf("D=%d L=%u blocks=%u strips=%u w=%u nb=%u\n", D, L, blocks, o.on, o.w, o.nb);
    }
    if (strips < 3) ++bad; // the shapes above include strip-mined ones (48^4, 64^4, 96^4, 256^3, 512^3)
    std::printf(bad ? "FAILED %d\n" : "PASSED\n", bad);
    return bad ? 1 : 0;
}
