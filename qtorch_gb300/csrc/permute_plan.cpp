// Host planning of the tiled index permutation (permute.h): which digits a
// tile spans and the offset tables the kernels (permute.cu) index.
#include <algorithm>

#include "permute.h"

namespace qtg {

bool permute_plan(int rank, const int32_t *perm, uint32_t elem_bytes, PermutePlan &p) {
    if (rank < 0 || rank > kPermMaxRank || (rank > 0 && !perm) || (elem_bytes != 8 && elem_bytes != 16)) return false;
    p = PermutePlan{};
    p.rank = (uint32_t) rank;
    p.elem_bytes = elem_bytes;
    int opos[kPermMaxRank];
    bool seen[kPermMaxRank] = {false};
    for (int i = 0; i < rank; i++) {
        if (perm[i] < 0 || perm[i] >= rank || seen[perm[i]]) return false;
        seen[perm[i]] = true;
        opos[perm[i]] = i;
    }
    // tile digits: X's lowest a and the X digits of Y's lowest b
    const int a = std::min(kPermLowDigits, rank), b = std::min(kPermLowDigits, rank);
    bool in_u[kPermMaxRank] = {false};
    for (int x = 0; x < a; x++) in_u[x] = true;
    for (int i = 0; i < b; i++) in_u[perm[i]] = true;
    // a tile of fewer digits (the permutation keeps low digits in place) takes
    // X's next-lowest digits too: 4096-element tiles keep the copies long
    int cnt = 0;
    for (int x = 0; x < rank; x++) cnt += in_u[x];
    for (int x = 0; x < rank && cnt < kPermMaxTileDigits; x++)
        if (!in_u[x]) {
            in_u[x] = true;
            cnt++;
        }
    int nu = 0;
    for (int x = 0; x < rank; x++)
        if (in_u[x]) p.u_in[nu++] = (uint8_t) x;   // ascending X order; the first a are 0..a-1
    p.nu = (uint32_t) nu;
    p.a = (uint32_t) a;
    p.b = (uint32_t) b;
    int nr = 0;
    for (int x = 0; x < rank; x++)
        if (!in_u[x]) {
            p.r_in[nr] = (uint8_t) x;
            p.r_out[nr] = (uint8_t) opos[x];
            nr++;
        }
    p.n_rest = (uint32_t) nr;
    p.n_tiles = 1ull << (2 * nr);
    // tile digits in ascending Y order (v[i] = tile digit); Y's lowest b come first
    int v[kPermMaxTileDigits];
    for (int j = 0; j < nu; j++) v[j] = j;
    std::sort(v, v + nu, [&](int x, int y) { return opos[p.u_in[x]] < opos[p.u_in[y]]; });
    const uint32_t hi_in = 1u << (2 * (nu - a)), hi_out = 1u << (2 * (nu - b)), lo_out = 1u << (2 * b);
    for (uint32_t h = 0; h < hi_in; h++) {
        uint32_t o = 0;
        for (int j = a; j < nu; j++) o += ((h >> (2 * (j - a))) & 3u) << (2 * p.u_in[j]);
        p.in_hi[h] = o;
    }
    for (uint32_t h = 0; h < hi_out; h++) {
        uint32_t o = 0, e = 0;
        for (int i = b; i < nu; i++) {
            const uint32_t dg = (h >> (2 * (i - b))) & 3u;
            o += dg << (2 * opos[p.u_in[v[i]]]);
            e += dg << (2 * v[i]);
        }
        p.out_hi[h] = o;
        p.e_hi[h] = (uint16_t) e;
    }
    for (uint32_t l = 0; l < lo_out; l++) {
        uint32_t e = 0;
        for (int i = 0; i < b; i++) e += ((l >> (2 * i)) & 3u) << (2 * v[i]);
        p.e_lo[l] = (uint16_t) e;
    }
    return true;
}

}  // namespace qtg
