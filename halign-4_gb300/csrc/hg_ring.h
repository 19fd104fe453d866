// hg_ring.h - the request-byte ring of the serving loop (hg_serve.cpp);
// host code only, no CUDA.
//
// Positions grow without bound and the byte at position p lives at offset
// p % cap.  A reservation never wraps: one that would cross the end of the
// buffer starts at the next lap instead, so every request's bytes are
// contiguous in memory.  Reservations are made in position order by one
// writer at a time and freed in position order (the loop frees up to its
// oldest unfiled request), so the live bytes are exactly [tail, head).
#pragma once

#include <cstdint>

namespace hg {

struct ByteRing {
    int64_t cap = 0;
    int64_t head = 0;       // end of the last reservation
    int64_t tail = 0;       // start of the oldest live byte
    int64_t published = 0;  // end of the last reservation handed to readers

    // Where len bytes would start after head.
    int64_t place(int64_t len) const
    {
        const int64_t off = head % cap;
        return len > 0 && off + len > cap ? head + (cap - off) : head;
    }
    // Whether len bytes can be reserved now (always, once the ring is
    // empty, for len <= cap / 2: the skipped end of a lap is below len).
    bool fits(int64_t len) const { return place(len) + len - tail <= cap; }
    // Reserves len bytes (fits(len) must hold) and returns their position.
    int64_t reserve(int64_t len)
    {
        const int64_t p = place(len);
        head = p + len;
        return p;
    }
    // The reservations made so far are readable (queued).
    void publish() { published = head; }
    // Frees every byte before pos, the position of the oldest live request.
    void release_before(int64_t pos) { tail = pos; }
    // Frees every published byte (no queued request is live).
    void release_all() { tail = published; }
    int64_t offset(int64_t pos) const { return pos % cap; }
    // Whether bytes at pos continue in memory a run that ends at end.
    bool continues(int64_t end, int64_t pos) const { return pos == end && end % cap != 0; }
};

}  // namespace hg
