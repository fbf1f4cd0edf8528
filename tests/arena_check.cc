// Randomised check of the serving loop's arena allocator
// (cusat_gb300/csrc/arena.h): blocks never overlap, never leave the range,
// usage and peak are exact, and releasing everything coalesces back to one
// free block.  Prints OK on success.
#include <stdio.h>
#include <stdlib.h>

#include <random>
#include <vector>

#include "arena.h"

int main()
{
    const size_t size = 1 << 20;
    cusat_internal::Arena a(size, 256);
    std::mt19937_64 rng(7);
    struct Blk { size_t off, n; };
    std::vector<Blk> live;
    size_t used = 0, peak = 0;
    for (int it = 0; it < 200000; it++) {
        if (live.empty() || rng() % 3 != 0) {
            const size_t n = 1 + rng() % 40000;
            size_t off;
            const bool ok = a.alloc(n, &off);
            const size_t need = a.round(n);
            if (ok) {
                if (off % 256 || off + need > size) { printf("FAIL range\n"); return 1; }
                for (const Blk& b : live)
                    if (off < b.off + a.round(b.n) && b.off < off + need) { printf("FAIL overlap\n"); return 1; }
                live.push_back({off, n});
                used += need;
                if (used > peak) peak = used;
            } else if (a.largest() >= need) {
                printf("FAIL refused a fitting block\n");
                return 1;
            }
        } else {
            const size_t k = rng() % live.size();
            a.release(live[k].off, live[k].n);
            used -= a.round(live[k].n);
            live[k] = live.back();
            live.pop_back();
        }
        if (a.used() != used || a.peak() != peak) { printf("FAIL accounting\n"); return 1; }
    }
    for (const Blk& b : live)
        a.release(b.off, b.n);
    if (a.used() != 0 || a.free_blocks() != 1 || a.largest() != size) { printf("FAIL coalesce\n"); return 1; }
    printf("OK\n");
    return 0;
}
