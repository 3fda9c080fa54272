// block_order.hpp -- the order in which the per-site stencil kernels (k_md_site, k_gauss_sweep) visit
// their blocks of 128 consecutive sites.
//
// In site order the blocks that run at the same time cover a slab of about (resident blocks x 128)
// sites, and a site's neighbour along the slowest direction lies L^(D-1) sites away.  Once that
// distance is several slabs (48^4 and above at D = 4, 256^3 at D = 3) the neighbour links read by one
// wave of blocks have left L2 before the wave that needs them again runs.  Strip-mining the sheets of
// constant (x_{D-2}, x_{D-1}) fixes the distance: the sheets are taken in strips of w consecutive
// x_{D-2}, x_{D-1} running inside a strip, so a neighbour along x_{D-1} lies w L^(D-2) sites of work
// away.  The order only permutes whole blocks (each still 128 consecutive sites, four whole tiles), so
// every site's arithmetic, and every result, is that of the site order; a block's residual partial
// keeps its site-order slot.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define LQ_HD __host__ __device__ __forceinline__
#else
#define LQ_HD inline
#endif

namespace lq {

struct BlockOrder {
    uint32_t on;    // 0: site order
    uint32_t nb;    // blocks per sheet of constant (x_{D-2}, x_{D-1}): L^(D-2) / block_sites
    uint32_t w;     // sheets per strip along x_{D-2} (divides L)
    uint32_t L;
};

// w = the largest divisor of L with w L^(D-2) <= reuse_sites; site order when that is L itself, when
// D < 3, or when a sheet is not a whole number of blocks
inline BlockOrder make_block_order(int D, uint32_t L, uint32_t block_sites, uint32_t reuse_sites) {
    BlockOrder o = {0, 1, L, L};
    if (D < 3 || L == 0) return o;
    uint64_t sheet = 1;
    for (int i = 0; i < D - 2; ++i) sheet *= L;
    if (sheet % block_sites != 0) return o;
    uint32_t w = 0;
    for (uint32_t d = 1; d <= L; ++d)
        if (L % d == 0 && (uint64_t)d * sheet <= reuse_sites) w = d;
    if (w == 0 || w == L) return o;
    o.on = 1;
    o.nb = (uint32_t)(sheet / block_sites);
    o.w = w;
    return o;
}

// the site-order index of the block that runs b-th
LQ_HD uint32_t block_at(const BlockOrder &o, uint32_t b) {
    if (!o.on) return b;
    const uint32_t j = b % o.nb, q = b / o.nb;       // block within the sheet, sheet in launch order
    const uint32_t r = q % o.w, q2 = q / o.w;          // x_{D-2} within the strip
    const uint32_t x_last = q2 % o.L, strip = q2 / o.L; // x_{D-1}, strip
    const uint32_t x_second = strip * o.w + r;
    return (x_last * o.L + x_second) * o.nb + j;
}

} // namespace lq
