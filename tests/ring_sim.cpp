// ring_sim.cpp - randomized check of the serving loop's request-byte ring
// (halign-4_gb300/csrc/hg_ring.h) against the way hg_serve.cpp drives it:
// one writer reserves, copies and publishes requests in order; micro-batches
// take the oldest queued requests and read them as runs of contiguous
// memory; batches finish in any order and the ring is freed up to the
// oldest unfinished request.  Checks that no request wraps, that every
// batch's runs hold exactly its requests' bytes, that no live byte is ever
// overwritten and that an empty ring always takes a request of up to
// cap / 2 bytes.  Usage: ring_sim <seed> <steps>; exit status 0 = pass.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <deque>
#include <random>
#include <vector>

#include "hg_ring.h"

namespace {

struct Req {
    int64_t pos, len;
    uint32_t seed;
    bool released = false;
};

uint8_t byte_of(uint32_t seed, int64_t i) { return (uint8_t)((seed * 2654435761u + (uint32_t)i * 40503u) >> 13); }

int fails = 0;
void check(bool ok, const char* what, long step)
{
    if (!ok && fails++ < 10) std::fprintf(stderr, "step %ld: %s\n", step, what);
}

}  // namespace

int main(int argc, char** argv)
{
    const uint32_t seed = argc > 1 ? (uint32_t)std::atoi(argv[1]) : 1;
    const long steps = argc > 2 ? std::atol(argv[2]) : 20000;
    std::mt19937_64 rng(seed);
    hg::ByteRing rb;
    rb.cap = 512 + (int64_t)(rng() % 4096);
    const int64_t max_len = rb.cap / 2;
    std::vector<uint8_t> mem((size_t)rb.cap, 0);
    std::deque<Req> reqs;  // id - base indexes it
    int64_t base = 0, rel = 0;
    std::deque<int64_t> pending;
    std::vector<std::vector<int64_t>> inflight;
    uint32_t next_seed = 1;
    auto advance = [&] {
        const int64_t end = base + (int64_t)reqs.size();
        while (rel < end && reqs[(size_t)(rel - base)].released) ++rel;
        if (rel < end) rb.release_before(reqs[(size_t)(rel - base)].pos);
        else rb.release_all();
        while (!reqs.empty() && reqs.front().released) reqs.pop_front(), ++base;  // results returned
    };
    for (long step = 0; step < steps; ++step) {
        const int op = (int)(rng() % 3);
        if (op == 0) {  // a burst: reserve what fits, copy, publish
            const int n = 1 + (int)(rng() % 6);
            std::vector<Req> burst;
            for (int k = 0; k < n; ++k) {
                const int64_t len = (rng() % 8 == 0) ? 0 : 1 + (int64_t)(rng() % (uint64_t)max_len);
                if (!rb.fits(len)) break;
                Req r{rb.reserve(len), len, next_seed++};
                check(rb.offset(r.pos) + r.len <= rb.cap, "request wraps", step);
                burst.push_back(r);
            }
            for (const Req& r : burst)  // (bounded: a wrapping request is reported above, not written past the end)
                for (int64_t i = 0; i < r.len && rb.offset(r.pos) + i < rb.cap; ++i)
                    mem[(size_t)(rb.offset(r.pos) + i)] = byte_of(r.seed, i);
            for (const Req& r : burst) {
                pending.push_back(base + (int64_t)reqs.size());
                reqs.push_back(r);
            }
            rb.publish();
            check(rb.head - rb.tail <= rb.cap, "live bytes exceed the ring", step);
        } else if (op == 1 && !pending.empty()) {  // admit the oldest as a micro-batch; read it as runs
            const int take = 1 + (int)(rng() % 8);
            std::vector<int64_t> ids;
            std::vector<std::pair<int64_t, int64_t>> runs;  // (offset, bytes)
            int64_t end = -1;
            std::vector<uint8_t> want;
            int64_t bytes = 0;  // a batch holds at most max_len bytes, as a context holds slot_bases
            while (!pending.empty() && (int)ids.size() < take) {
                const int64_t id = pending.front();
                const Req& r = reqs[(size_t)(id - base)];
                if (!ids.empty() && bytes + r.len > max_len) break;
                pending.pop_front();
                ids.push_back(id);
                bytes += r.len;
                for (int64_t i = 0; i < r.len; ++i) want.push_back(byte_of(r.seed, i));
                if (r.len == 0) continue;
                if (rb.continues(end, r.pos)) runs.back().second += r.len;
                else runs.push_back({rb.offset(r.pos), r.len});
                end = r.pos + r.len;
            }
            std::vector<uint8_t> got;
            for (const auto& ru : runs) {
                check(ru.first + ru.second <= rb.cap, "run passes the end of the ring", step);
                for (int64_t i = 0; i < ru.second && ru.first + i < rb.cap; ++i) got.push_back(mem[(size_t)(ru.first + i)]);
            }
            check(got == want, "a batch's runs differ from its requests' bytes", step);
            check(runs.size() <= 2, "more than two runs for one batch", step);
            inflight.push_back(ids);
        } else if (!inflight.empty()) {  // a batch finishes (any of them); its requests are filed
            const size_t b = (size_t)(rng() % inflight.size());
            for (const int64_t id : inflight[b]) {
                Req& r = reqs[(size_t)(id - base)];
                bool intact = true;
                for (int64_t i = 0; i < r.len; ++i)
                    intact = intact && rb.offset(r.pos) + i < rb.cap && mem[(size_t)(rb.offset(r.pos) + i)] == byte_of(r.seed, i);
                check(intact, "a live request's bytes were overwritten", step);
                r.released = true;
            }
            inflight.erase(inflight.begin() + (long)b);
            advance();
            if (pending.empty() && inflight.empty())
                check(rb.fits(max_len), "an empty ring refuses a request of cap / 2 bytes", step);
        }
    }
    std::printf("ring_sim seed %u cap %lld: %ld steps, %u requests, %d failures\n", seed, (long long)rb.cap, steps,
                next_seed - 1, fails);
    return fails ? 1 : 0;
}
