// Checks the host-buffer page arithmetic (csrc/host_pages.hpp) against its
// rules on many buffer placements, group sizes and page sizes:
//  - registered ranges (whole pages, chunk by chunk) lie inside the buffer,
//    are page-aligned and never overlap;
//  - each group's pieces tile its bytes exactly, in order;
//  - a chunk piece of group k lies in one chunk j <= k (locked before the
//    group's copy is issued); head and tail pieces lie in the buffer's
//    partial end pages, each shorter than a page.
#include "host_pages.hpp"

#include <cstdio>
#include <random>

using namespace bcg;

static int fail(const char* what, unsigned long long a, unsigned long long b) {
    std::printf("FAIL %s (%llu, %llu)\n", what, a, b);
    return 1;
}

int main() {
    std::mt19937_64 rng(7);
    std::vector<CopyPiece> pieces;
    long checked = 0;
    for (int trial = 0; trial < 200000; ++trial) {
        const uintptr_t page = (rng() & 1) ? 4096 : 65536;
        const uintptr_t base = (uintptr_t(1) << 30) + (rng() % (1u << 22)) * 4;
        const size_t steps[] = {4, 64, 4096, 16384, 65536 * 3 + 4, 1000000, 57671680};
        const size_t step = steps[rng() % 7];
        const size_t groups = 1 + rng() % 40;
        size_t total = step * groups;
        if (rng() & 1) total -= 4 * (rng() % (step / 4));
        if (total == 0) continue;
        const ChunkPlan c(base, total, step, page);
        // Registered chunks.
        uintptr_t prev = c.span.lo;
        for (size_t k = 0; k < c.chunks; ++k) {
            const uintptr_t lo = c.bound(k), hi = c.bound(k + 1);
            if (lo % page || hi % page) return fail("unaligned chunk", lo, hi);
            if (hi < lo || lo < prev) return fail("chunks out of order", lo, prev);
            if (hi > lo && (lo < base || hi > base + total)) return fail("chunk outside the buffer", lo, hi);
            prev = hi;
        }
        if (c.span.lo - base >= page && c.span.lo != base) return fail("head of a page or more", c.span.lo, base);
        if (base + total - c.span.hi >= page && c.span.hi > c.span.lo) return fail("tail of a page or more", c.span.hi, base);
        // Group pieces.
        for (size_t k = 0; k < c.chunks; ++k) {
            group_pieces(c, k, pieces);
            uintptr_t pos = base + k * step;
            const uintptr_t end = std::min(base + total, pos + step);
            for (const CopyPiece& p : pieces) {
                if (p.lo != pos || p.hi <= p.lo) return fail("pieces do not tile the group", p.lo, pos);
                pos = p.hi;
                if (p.kind == PieceKind::chunk) {
                    if (p.chunk > k) return fail("piece in a chunk not yet locked", p.chunk, k);
                    if (p.lo < c.bound(p.chunk) || p.hi > c.bound(p.chunk + 1)) return fail("piece spans chunks", p.lo, p.hi);
                } else if (p.kind == PieceKind::head) {
                    if (p.hi > c.span.lo && c.span.hi > c.span.lo) return fail("head past the first whole page", p.hi, c.span.lo);
                    if (p.hi - base >= page && c.span.hi > c.span.lo) return fail("head longer than a page", p.hi, base);
                } else {
                    if (p.lo < c.span.hi) return fail("tail before the last whole page", p.lo, c.span.hi);
                    if (base + total - p.lo >= page) return fail("tail longer than a page", p.lo, base);
                }
                ++checked;
            }
            if (pos != end) return fail("pieces short of the group", pos, end);
        }
        // Whole pages of an arbitrary run.
        const size_t run = 1 + rng() % (3 * page);
        const PageSpan w = whole_pages(base, run, page);
        if (w.hi > w.lo && (w.lo < base || w.hi > base + run || w.lo % page || w.hi % page))
            return fail("whole pages outside the run", w.lo, w.hi);
    }
    std::printf("ok %ld pieces\n", checked);
    return 0;
}
