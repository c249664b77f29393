// CPU emulation of the tiled index permutation (qtorch_gb300/csrc/permute.cu)
// for the host tests: for random ranks and permutations it asks the library's
// permute_plan for the tiling, then walks every tile the way the kernel's
// threads do -- the 16-byte pair loads along X's contiguous digits (8-byte
// elements) or single loads, the swizzled shared-memory slots, the pair
// stores along Y's contiguous digits -- checking every index against its
// buffer, the 16-byte alignment of every pair access, that every shared slot
// and every output element is written exactly once, and every output against
// the index map (digit i of Y's index = digit perm[i] of X's).  No GPU.
//
//   permute_emulator <seed> <cases>      prints "ok <checked>" or the first failure
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "../qtorch_gb300/csrc/permute.h"

using namespace qtg;

static uint32_t swz(uint32_t e) { return e ^ (((e >> 4) ^ (e >> 8)) & 15u); }

static bool fail(const char *what, int rank, const std::vector<int32_t> &perm) {
    std::printf("FAIL %s rank %d perm", what, rank);
    for (int v : perm) std::printf(" %d", v);
    std::printf("\n");
    return false;
}

static bool check_case(int rank, const std::vector<int32_t> &perm, uint32_t elem) {
    PermutePlan p;
    if (!permute_plan(rank, perm.data(), elem, p)) return fail("plan refused", rank, perm);
    const uint64_t N = 1ull << (2 * rank);
    const uint32_t n = 1u << (2 * p.nu), ma = (1u << (2 * p.a)) - 1u, mb = (1u << (2 * p.b)) - 1u;
    if (p.nu > (uint32_t) kPermMaxTileDigits || (p.a + 3 < p.nu) || (p.b + 3 < p.nu) || p.b > 3 || p.a > 3)
        return fail("table sizes", rank, perm);
    if ((uint64_t) n * p.n_tiles != N) return fail("tiles do not cover the tensor", rank, perm);
    std::vector<uint64_t> out(N, ~0ull);
    std::vector<int> tile_slot(n);
    std::vector<uint64_t> tile(n);
    const bool pairs = elem == 8 && n >= 2;
    for (uint64_t t = 0; t < p.n_tiles; t++) {
        uint64_t bi = 0, bo = 0;
        for (uint32_t j = 0; j < p.n_rest; j++) {
            const uint64_t dg = (t >> (2 * j)) & 3ull;
            bi += dg << (2 * p.r_in[j]);
            bo += dg << (2 * p.r_out[j]);
        }
        std::fill(tile_slot.begin(), tile_slot.end(), 0);
        for (uint32_t e = 0; e < n; e += pairs ? 2 : 1) {
            if ((e >> (2 * p.a)) >= 64) return fail("in_hi index", rank, perm);
            const uint64_t o = bi + (e & ma) + p.in_hi[e >> (2 * p.a)];
            const uint32_t k = pairs ? 2 : 1;
            if (o + k > N) return fail("load out of bounds", rank, perm);
            if (pairs && (o & 1)) return fail("pair load not 16-byte aligned", rank, perm);
            for (uint32_t q = 0; q < k; q++) {
                const uint32_t s = swz(e + q);
                if (s >= n) return fail("shared slot out of range", rank, perm);
                if (tile_slot[s]++) return fail("shared slot written twice", rank, perm);
                tile[s] = o + q;
            }
        }
        for (uint32_t f = 0; f < n; f += pairs ? 2 : 1) {
            if ((f >> (2 * p.b)) >= 64 || (f & mb) + (pairs ? 1 : 0) >= 64) return fail("table index", rank, perm);
            const uint32_t hi = p.e_hi[f >> (2 * p.b)];
            const uint64_t o = bo + (f & mb) + p.out_hi[f >> (2 * p.b)];
            const uint32_t k = pairs ? 2 : 1;
            if (o + k > N) return fail("store out of bounds", rank, perm);
            if (pairs && (o & 1)) return fail("pair store not 16-byte aligned", rank, perm);
            for (uint32_t q = 0; q < k; q++) {
                const uint32_t e = (uint32_t) p.e_lo[(f & mb) + q] + hi;
                if (e >= n) return fail("tile element out of range", rank, perm);
                if (out[o + q] != ~0ull) return fail("output written twice", rank, perm);
                out[o + q] = tile[swz(e)];
            }
        }
    }
    for (uint64_t y = 0; y < N; y++) {
        uint64_t x = 0;
        for (int i = 0; i < rank; i++) x += ((y >> (2 * i)) & 3ull) << (2 * perm[i]);
        if (out[y] != x) return fail("wrong element", rank, perm);
    }
    return true;
}

int main(int argc, char **argv) {
    const unsigned seed = argc > 1 ? (unsigned) std::atoi(argv[1]) : 1;
    const int cases = argc > 2 ? std::atoi(argv[2]) : 50;
    std::mt19937 g(seed);
    int checked = 0;
    for (int c = 0; c < cases; c++) {
        const int rank = (int) (g() % 11);   // 0..10
        std::vector<int32_t> perm(rank);
        for (int i = 0; i < rank; i++) perm[i] = i;
        const int kind = c % 4;
        if (kind == 1) std::reverse(perm.begin(), perm.end());
        if (kind >= 2) std::shuffle(perm.begin(), perm.end(), g);
        for (uint32_t elem : {8u, 16u}) {
            if (!check_case(rank, perm, elem)) return 1;
            checked++;
        }
    }
    // a permutation is refused when it is not one
    PermutePlan p;
    const int32_t bad[3] = {0, 0, 1};
    if (permute_plan(3, bad, 8, p)) {
        std::printf("FAIL accepted a non-permutation\n");
        return 1;
    }
    std::printf("ok %d\n", checked);
    return 0;
}
