// The receive chain's split copy (cusat_gb300/csrc/copy_crew.h) on its own:
// crews created and used at once (a job published before the helpers run),
// copies of every size class byte-exact, reuse across many jobs, sleep and
// wake after quiet intervals, destruction with idle and sleeping helpers.
// Prints "OK" and exits 0 on success.
#include <stdio.h>

#include <random>
#include <vector>

#include "copy_crew.h"

using cusat_internal::CopyCrew;

static int check(CopyCrew& crew, std::mt19937& rng, size_t bytes)
{
    std::vector<uint8_t> src(bytes), dst(bytes + 64, 0xA5);
    for (auto& b : src)
        b = (uint8_t)rng();
    crew.copy(dst.data(), src.data(), bytes);
    for (size_t i = 0; i < bytes; i++)
        if (dst[i] != src[i])
            return 1;
    for (size_t i = bytes; i < bytes + 64; i++)
        if (dst[i] != 0xA5)
            return 1;  // nothing written past the end
    return 0;
}

int main()
{
    std::mt19937 rng(1);
    const size_t sizes[] = {0, 1, 100, 32767, 32768, 64800, 172800, 172801, 1 << 20, 3000017};
    for (int round = 0; round < 200; round++) {
        CopyCrew crew(1 + round % 4);  // used right away: the helpers may not have started
        for (size_t b : sizes)
            if (check(crew, rng, b)) {
                printf("FAIL copy of %zu bytes, %d helpers\n", b, 1 + round % 4);
                return 1;
            }
    }
    CopyCrew crew(3);
    for (int i = 0; i < 2000; i++)
        if (check(crew, rng, 16384 + rng() % 400000)) {
            printf("FAIL stream of copies\n");
            return 1;
        }
    for (int i = 0; i < 3; i++) {
        std::this_thread::sleep_for(std::chrono::milliseconds(20));  // helpers go to sleep
        if (check(crew, rng, 172800)) {
            printf("FAIL copy after a quiet interval\n");
            return 1;
        }
    }
    CopyCrew none(0);
    if (check(none, rng, 172800)) {
        printf("FAIL copy without helpers\n");
        return 1;
    }
    printf("OK\n");
    return 0;
}
