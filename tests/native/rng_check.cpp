// Prints, for each u64 read from stdin, the library's small_seed(h) state words, its first four
// next_u64 outputs and small_first_u64(h) (the emptiness-test shortcut), as decimal numbers on one
// line; then one line with the state of small_seed_zero() (the all-zero-seed remap).
#include <cinttypes>
#include <cstdio>
#include "fg_rng.cuh"

int main() {
    unsigned long long h;
    while (std::scanf("%llu", &h) == 1) {
        fg::Xoshiro x = fg::small_seed(h);
        std::printf("%" PRIu64 " %" PRIu64 " %" PRIu64 " %" PRIu64, x.s0, x.s1, x.s2, x.s3);
        for (int k = 0; k < 4; k++) std::printf(" %" PRIu64, x.next());
        std::printf(" %" PRIu64 "\n", fg::small_first_u64(h));
    }
    fg::Xoshiro z = fg::small_seed_zero();
    std::printf("%" PRIu64 " %" PRIu64 " %" PRIu64 " %" PRIu64 "\n", z.s0, z.s1, z.s2, z.s3);
    return 0;
}
