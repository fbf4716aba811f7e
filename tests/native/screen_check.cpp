// The emptiness-bitmask identities of the sparse pass, checked on the host with the library's own
// header (fg_rng.cuh):
//  1. first_draw_screen(h, screen_bound(t)) == ((small_first_u64(h) >> 11) > t) for every hash h whose
//     seed words 1, 2, 7, 8 are not all zero, on thresholds around each h's own draw and at the edges
//     (negative, 0, 2^53 - 2, 2^53 - 1, 2^53);
//  2. rotl64(base + r, 41) + phi == rotl64(base, 41) + phi + r * 2^41 for r < 32 whenever adding r carries
//     nothing out of base's low 23 bits (the row-hash input of a bitmask word).
// Prints "checked mismatches" for each part.
#include <cstdio>
#include <cstdint>

#include "fg_rng.cuh"

using namespace fg;

int main() {
    uint64_t st = 12345;
    long long checked = 0, bad = 0;
    for (int n = 0; n < 200000; n++) {
        st += kPhi;
        const uint64_t h = fmix64(st);
        const long long v = (long long)(small_first_u64(h) >> 11);
        const long long ts[] = {-5, -1, 0, 1, v - 2, v - 1, v, v + 1, v + 2, (1ll << 53) - 2, (1ll << 53) - 1,
                                1ll << 53, (long long)(0.962 * (double)(1ll << 53))};
        for (long long t : ts) {
            const bool want = v > t;
            const bool got = first_draw_screen(h, screen_bound(t));
            checked++;
            if (want != got) bad++;
        }
    }
    std::printf("%lld %lld\n", checked, bad);
    long long checked2 = 0, bad2 = 0;
    st = 777;
    for (int n = 0; n < 200000; n++) {
        st += kPhi;
        const uint64_t base = fmix64(st);
        if ((base & 0x7FFFFFull) > 0x7FFFFFull - 31) continue;
        const uint64_t c0 = rotl64(base, 41) + kPhi;
        for (uint64_t r = 0; r < 32; r++) {
            checked2++;
            if (rotl64(base + r, 41) + kPhi != c0 + (r << 41)) bad2++;
        }
    }
    std::printf("%lld %lld\n", checked2, bad2);
    return 0;
}
