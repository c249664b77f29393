// CPU emulation of the streaming kernel (qtorch_gb300/csrc/stream.cu) for the
// host tests: for random contraction steps of the shapes the kernel takes, it
// asks the library's stream_plan for the tiling and then walks every tile the
// way the kernel's threads do -- the bulk-copy runs of the large operand, each
// thread's loop over its elements of the tile with its sums kept across the
// chunks of a work item, the reduction over the summed digits among wires 0-3
// (shuffles or staging) and the write-back to C -- checking every
// index against its buffer, that every output is written exactly once, and
// every output against a direct evaluation of the contraction.  No GPU.
//
//   stream_emulator <seed> <cases>      prints "ok <checked> <planned>" or the first failure
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

#include "../qtorch_gb300/csrc/stream.h"

using namespace qtg;
using cf = std::complex<float>;

// A step as ContractNodes forms it: C = A's free wires in A order, then B's;
// summed pairs at random wires of both operands (digit i of k <-> pair n-1-i).
// With shuffle_c the free wires take C's digits in a random order (as
// qt_contract_pair allows).
static void random_step(std::mt19937 &g, int rA, int rB, int nSum, bool shuffle_c, StepDesc &d) {
    std::vector<int> wa(rA), wb(rB);
    for (int i = 0; i < rA; i++) wa[i] = i;
    for (int i = 0; i < rB; i++) wb[i] = i;
    std::shuffle(wa.begin(), wa.end(), g);
    std::shuffle(wb.begin(), wb.end(), g);
    std::vector<bool> sa(rA, false), sb(rB, false);
    d = StepDesc{};
    d.rA = (uint8_t) rA;
    d.rB = (uint8_t) rB;
    d.nSum = (uint8_t) nSum;
    for (int j = 0; j < nSum; j++) {
        sa[wa[j]] = true;
        sb[wb[j]] = true;
        d.posAs[nSum - 1 - j] = (uint8_t) wa[j];
        d.posBs[nSum - 1 - j] = (uint8_t) wb[j];
    }
    int c = 0;
    for (int w = 0; w < rA; w++)
        if (!sa[w]) {
            d.cA[c] = (uint8_t) w;
            d.cB[c++] = kNoWire;
        }
    d.fA = (uint8_t) c;
    for (int w = 0; w < rB; w++)
        if (!sb[w]) {
            d.cB[c] = (uint8_t) w;
            d.cA[c++] = kNoWire;
        }
    d.fB = (uint8_t) (c - d.fA);
    d.nFree = (uint8_t) c;
    if (shuffle_c) {
        std::vector<int> perm(c);
        for (int i = 0; i < c; i++) perm[i] = i;
        std::shuffle(perm.begin(), perm.end(), g);
        uint8_t ca[kMaxWires], cb[kMaxWires];
        for (int i = 0; i < c; i++) {
            ca[i] = d.cA[perm[i]];
            cb[i] = d.cB[perm[i]];
        }
        for (int i = 0; i < c; i++) {
            d.cA[i] = ca[i];
            d.cB[i] = cb[i];
        }
    }
}

// one step: returns an empty string or what went wrong
static std::string emulate(const StepDesc &d, const StreamStep &p, std::mt19937 &g) {
    const uint64_t nA = 1ull << (2 * d.rA), nB = 1ull << (2 * d.rB), nC = 1ull << (2 * d.nFree);
    std::uniform_real_distribution<float> u(-1.f, 1.f);
    std::vector<cf> A(nA), B(nB), C(nC, cf(NAN, NAN));
    for (auto &x : A) x = cf(u(g), u(g));
    for (auto &x : B) x = cf(u(g), u(g));
    const std::vector<cf> &L = p.l_is_b ? B : A, &S = p.l_is_b ? A : B;
    const uint32_t NSF = 1u << (2 * p.nsfp), G = 1u << (2 * p.go), H = 1u << (2 * p.ho);
    const uint32_t tile_elems = 1u << (2 * (4 + p.go + p.ho));
    const uint32_t T = kStreamThreads, M = G * NSF;
    if (tile_elems > kStreamMaxTile || M > kStreamMaxStage || p.s_elems != S.size()) return "region sizes";
    if (p.run_elems * p.n_runs != tile_elems || p.run_elems < 256) return "runs";
    if (p.n_pass > 1 && p.n_chunks > 1) return "passes with chunks";
    // S's shared-memory image: element e at sum of digit_w(e) * s_unit[w];
    // every slot written at most once, in-pass blocks 16-byte aligned
    if (p.s_store > 8192) return "S image size";
    std::vector<cf> Simg(p.s_store, cf(NAN, NAN));
    std::vector<int> s_hits(p.s_store, 0);
    for (uint32_t e = 0; e < p.s_elems; e++) {
        uint32_t dst = 0;
        for (int w = 0; w < kStreamMaxSmallRank; w++) dst += ((e >> (2 * w)) & 3u) * p.s_unit[w];
        if (dst >= p.s_store) return "S image index";
        if (s_hits[dst]++) return "S image slot written twice";
        Simg[dst] = S[e];
    }
    std::vector<int> written(nC, 0);
    std::vector<cf> tile(tile_elems);
    // acc[pass][tid][i], i = g NSF + f, kept across the chunks of a work item
    std::vector<std::vector<std::vector<cf>>> acc(p.n_pass, std::vector<std::vector<cf>>(T, std::vector<cf>(M)));
    auto pass_offsets = [&](uint32_t pass, uint32_t &s_p, uint64_t &c_p) {
        s_p = 0;
        c_p = 0;
        for (uint32_t j = p.nsfp; j < p.nsf; j++) {
            const uint32_t dg = (pass >> (2 * (j - p.nsfp))) & 3u;
            s_p += dg * p.s_unit[p.sf_w[j]];
            c_p += (uint64_t) dg << (2 * p.sf_cd[j]);
        }
    };
    for (uint32_t item = 0; item < p.n_items; item++) {
        for (auto &a : acc)
            for (auto &v : a) std::fill(v.begin(), v.end(), cf(0.f, 0.f));
        for (uint32_t chunk = 0; chunk < p.n_chunks; chunk++) {
            // bulk copies
            uint64_t lbase = 0;
            for (uint32_t j = 0; j < p.n_item_d; j++) lbase += (uint64_t) ((item >> (2 * j)) & 3u) << (2 * p.item_lw[j]);
            for (uint32_t j = 0; j < p.n_chunk_d; j++) lbase += (uint64_t) ((chunk >> (2 * j)) & 3u) << (2 * p.chunk_lw[j]);
            for (uint32_t r = 0; r < p.n_runs; r++) {
                uint64_t off = lbase;
                for (uint32_t j = 0; j < p.n_run_d; j++) off += (uint64_t) ((r >> (2 * j)) & 3u) << (2 * p.run_lw[j]);
                if ((off * 8) % 16) return "bulk copy alignment";
                if (off + p.run_elems > L.size()) return "bulk copy beyond L";
                for (uint32_t e = 0; e < p.run_elems; e++) tile[(uint64_t) r * p.run_elems + e] = L[off + e];
            }
            uint32_t s_c = 0;
            for (uint32_t j = 0; j < p.n_chunk_d; j++) s_c += ((chunk >> (2 * j)) & 3u) * p.s_unit[p.chunk_sw[j]];
            for (uint32_t pass = 0; pass < p.n_pass; pass++) {
                uint32_t s_p;
                uint64_t c_p;
                pass_offsets(pass, s_p, c_p);
                for (uint32_t tid = 0; tid < T; tid++) {
                    uint32_t s_lo = 0;
                    for (int w = 0; w < 4; w++)
                        if (p.lo_summed[w]) s_lo += ((tid >> (2 * w)) & 3u) * p.s_unit[p.lo_other[w]];
                    for (uint32_t gg = 0; gg < G; gg++) {
                        uint32_t tg = tid;
                        for (uint32_t j = 0; j < p.go; j++) tg += ((gg >> (2 * j)) & 3u) << (2 * p.g_pos[j]);
                        for (uint32_t h = 0; h < H; h++) {
                            uint32_t th = tg, sh = s_c + s_p + s_lo;
                            for (uint32_t j = 0; j < p.ho; j++) {
                                const uint32_t dg = (h >> (2 * j)) & 3u;
                                th += dg << (2 * p.h_pos[j]);
                                sh += dg * p.s_unit[p.h_sw[j]];
                            }
                            if (th >= tile_elems) return "tile index";
                            // the kernel loads the block's NSF values as 16-byte pairs
                            if (NSF > 1 && (sh % 2)) return "S block not 16-byte aligned";
                            for (uint32_t f = 0; f < NSF; f++) {
                                if (sh + f >= p.s_store || !s_hits[sh + f]) return "small operand index";
                                acc[pass][tid][gg * NSF + f] += tile[th] * Simg[sh + f];
                            }
                        }
                    }
                }
            }
        }
        uint64_t cbase = 0;
        for (uint32_t j = 0; j < p.n_item_d; j++) cbase += (uint64_t) ((item >> (2 * j)) & 3u) << (2 * p.item_cd[j]);
        const uint32_t LM = M >= 16 ? 4 : M >= 4 ? 2 : 0;
        const uint32_t b0 = p.lo_summed[0] ? 0u : 2u, nb = 2u * (p.lo_summed[0] + p.lo_summed[1]);
        for (uint32_t pass = 0; pass < p.n_pass; pass++) {
            uint32_t s_p;
            uint64_t cpass;
            pass_offsets(pass, s_p, cpass);
            cpass += cbase;
            // butterfly reduce-scatter over the summed lane bits of wires 0/1, then all-reduce
            auto flat = acc[pass];
            std::vector<uint32_t> base(T, 0);
            std::vector<bool> owner(T, true);
            for (uint32_t k = 0; k < LM && k < nb; k++) {
                const uint32_t mask = 1u << (b0 + k), half = M >> (k + 1);
                if (mask >= 32) return "shuffle beyond a warp";
                auto next = flat;
                for (uint32_t tid = 0; tid < T; tid++) {
                    const bool hi = (tid & mask) != 0;
                    const uint32_t q = tid ^ mask;
                    for (uint32_t i = 0; i < half; i++) {
                        const cf send_q = !hi ? flat[q][i] : flat[q][i + half];
                        next[tid][i] = (hi ? flat[tid][i + half] : flat[tid][i]) + send_q;
                    }
                    if (hi) base[tid] += half;
                }
                flat = next;
            }
            const uint32_t m_left = M >> std::min(nb, LM);
            for (uint32_t k = LM; k < nb; k++) {
                const uint32_t mask = 1u << (b0 + k);
                if (mask >= 32) return "shuffle beyond a warp";
                auto next = flat;
                for (uint32_t tid = 0; tid < T; tid++) {
                    next[tid][0] = flat[tid][0] + flat[tid ^ mask][0];
                    if (tid & mask) owner[tid] = false;
                }
                flat = next;
            }
            const uint32_t n_out = 1u << (2 * p.n_dout);
            std::vector<cf> ostage(p.staged ? n_out : 0, cf(0.f, 0.f));
            std::vector<int> staged_hits(p.staged ? n_out : 0, 0);
            for (uint32_t tid = 0; tid < T; tid++) {
                if (!owner[tid]) continue;
                uint32_t c_lo = 0, st_lo = 0;
                for (int w = 0; w < 4; w++)
                    if (!p.lo_summed[w]) {
                        const uint32_t dg = (tid >> (2 * w)) & 3u;
                        c_lo += dg << (2 * p.lo_other[w]);
                        st_lo += dg << (2 * p.lo_rank[w]);
                    }
                for (uint32_t j = 0; j < m_left; j++) {
                    const uint32_t idx = base[tid] + j, gg = idx / NSF, f = idx % NSF;
                    if (idx >= M) return "reduce-scatter index";
                    if (p.staged) {
                        uint32_t u = st_lo;
                        for (uint32_t jj = 0; jj < p.go; jj++) u += ((gg >> (2 * jj)) & 3u) << (2 * p.g_rank[jj]);
                        for (uint32_t jj = 0; jj < p.nsfp; jj++) u += ((f >> (2 * jj)) & 3u) << (2 * p.sf_rank[jj]);
                        if (u >= n_out) return "staging index";
                        ostage[u] += flat[tid][j];
                        staged_hits[u]++;
                    } else {
                        uint64_t coff = cpass + c_lo;
                        for (uint32_t jj = 0; jj < p.go; jj++) coff += (uint64_t) ((gg >> (2 * jj)) & 3u) << (2 * p.g_cd[jj]);
                        for (uint32_t jj = 0; jj < p.nsfp; jj++) coff += (uint64_t) ((f >> (2 * jj)) & 3u) << (2 * p.sf_cd[jj]);
                        if (coff >= nC) return "C index";
                        written[coff]++;
                        C[coff] = flat[tid][j];
                    }
                }
            }
            if (p.staged) {
                const uint32_t expect = p.klo_mode == 2 ? 1u << (2 * (p.n_klo - nb / 2)) : 1u;
                for (uint32_t u = 0; u < n_out; u++)
                    if ((uint32_t) staged_hits[u] != expect) return "staging coverage";
                for (uint32_t u = 0; u < n_out; u++) {
                    uint64_t coff = cpass;
                    for (uint32_t r = 0; r < p.n_dout; r++) coff += (uint64_t) ((u >> (2 * r)) & 3u) << (2 * p.dout_cd[r]);
                    if (p.out_run >= 1 && (u & 1u) == 0 && (coff & 1u)) return "16-byte store alignment";
                    if (coff >= nC) return "C index";
                    written[coff]++;
                    C[coff] = ostage[u];
                }
            }
        }
    }
    for (uint64_t c = 0; c < nC; c++)
        if (written[c] != 1) return "C coverage";
    // direct evaluation
    const uint64_t KK = 1ull << (2 * d.nSum);
    for (uint64_t c = 0; c < nC; c++) {
        uint64_t oa, ob;
        scatter_c(c, d, oa, ob);
        std::complex<double> want = 0.0;
        for (uint64_t k = 0; k < KK; k++)
            want += std::complex<double>(A[oa + scatter_digits(k, d.posAs, d.nSum)]) *
                    std::complex<double>(B[ob + scatter_digits(k, d.posBs, d.nSum)]);
        if (std::abs(std::complex<double>(C[c]) - want) > 1e-5 * (1.0 + std::sqrt((double) KK)))
            return "value at output " + std::to_string(c);
    }
    return "";
}

int main(int argc, char **argv) {
    const unsigned seed = argc > 1 ? (unsigned) std::atoi(argv[1]) : 1;
    const int cases = argc > 2 ? std::atoi(argv[2]) : 200;
    std::mt19937 g(seed);
    // (rank A, rank B, summed) of the steps the kernel meets, small enough to check directly
    const int shapes[][3] = {{10, 3, 1}, {3, 10, 1}, {10, 4, 3}, {4, 10, 2}, {9, 5, 2}, {5, 9, 2}, {10, 1, 1},
                             {1, 10, 1}, {9, 2, 1}, {8, 6, 4}, {6, 8, 3}, {9, 5, 4}, {8, 4, 4}, {10, 2, 2},
                             {8, 3, 3}, {9, 6, 5}, {11, 4, 3}, {8, 5, 1}, {9, 3, 2}, {10, 6, 6}};
    const int n_shapes = sizeof shapes / sizeof shapes[0];
    int checked = 0, planned = 0;
    for (int i = 0; i < cases; i++) {
        const int *sh = shapes[i % n_shapes];
        StepDesc d;
        random_step(g, sh[0], sh[1], sh[2], (i / n_shapes) % 2 == 1, d);
        StreamStep p;
        if (!stream_plan(d, p)) continue;
        planned++;
        const std::string err = emulate(d, p, g);
        if (!err.empty()) {
            std::printf("fail case %d shape %d %d %d: %s\n", i, sh[0], sh[1], sh[2], err.c_str());
            return 1;
        }
        checked++;
    }
    std::printf("ok %d %d\n", checked, planned);
    return 0;
}
