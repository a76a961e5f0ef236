// Page arithmetic of the host-buffer path (no CUDA here, so that the host
// tests can check it on its own): which pages of a caller's buffer may be
// registered, the chunks an input buffer is locked in, and how one group's
// copy is cut.
//
// Only pages that lie wholly inside a buffer are ever registered.
// Registering an unaligned range locks the whole pages around it, taking in
// the neighbouring bytes of other buffers; a copy may not span two
// registrations, and a copy that starts in a registered page must stay in
// that registration.  So a group's bytes are cut into: the part in the
// buffer's partial first page (head), parts that each lie in one chunk of
// whole pages, and the part in the buffer's partial last page (tail).
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <vector>

namespace bcg {

// The whole pages of [p, p + bytes): [lo, hi), empty (lo == hi) when no page
// lies wholly inside.
struct PageSpan {
    uintptr_t lo = 0, hi = 0;
};

inline PageSpan whole_pages(uintptr_t p, size_t bytes, uintptr_t page) {
    PageSpan s;
    s.lo = (p + page - 1) & ~(page - 1);
    s.hi = std::max(s.lo, (p + bytes) & ~(page - 1));
    return s;
}

// An input buffer of `total` bytes at `base`, read in groups of `step` bytes
// (the last may be shorter).  Chunk k covers [bound(k), bound(k + 1)): the
// whole pages from the first page boundary at or after group k's start, so
// that group k's bytes lie in chunks 0..k and the partial end pages.
struct ChunkPlan {
    uintptr_t base = 0, page = 1;
    size_t total = 0, step = 1, chunks = 0;
    PageSpan span;

    ChunkPlan() = default;
    ChunkPlan(uintptr_t base_, size_t total_, size_t step_, uintptr_t page_)
        : base(base_), page(page_), total(total_), step(step_), chunks((total_ + step_ - 1) / step_),
          span(whole_pages(base_, total_, page_)) {}

    uintptr_t bound(size_t k) const {
        if (k == 0) return span.lo;
        if (k >= chunks) return span.hi;
        const uintptr_t x = (base + k * step + page - 1) & ~(page - 1);
        return std::min(std::max(x, span.lo), span.hi);
    }
};

enum class PieceKind { head, chunk, tail };

struct CopyPiece {
    uintptr_t lo, hi;   // host addresses
    PieceKind kind;
    size_t chunk;       // for kind == chunk
};

// The pieces of group k's bytes in address order: head, chunk pieces, tail
// (each only where non-empty).  Together they tile the group exactly.
inline void group_pieces(const ChunkPlan& c, size_t k, std::vector<CopyPiece>& out) {
    out.clear();
    const uintptr_t b = c.base + k * c.step;
    const uintptr_t e = std::min(c.base + c.total, b + c.step);
    if (b < std::min(e, c.span.lo)) out.push_back({b, std::min(e, c.span.lo), PieceKind::head, 0});
    for (size_t j = 0; j < c.chunks && j <= k; ++j) {
        const uintptr_t x = std::max(b, c.bound(j)), y = std::min(e, c.bound(j + 1));
        if (y > x) out.push_back({x, y, PieceKind::chunk, j});
    }
    const uintptr_t t = std::max(b, c.span.hi);
    if (t < e) out.push_back({t, e, PieceKind::tail, 0});
}

}  // namespace bcg
