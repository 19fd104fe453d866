/* Equivalence check for the small-tier DP arithmetic.
 *
 * For segments the band never binds, every cell the gap-fill DP reads is an
 * in-band cell, and the reference's difference encoding keeps u, v in [0, 21],
 * x, y in [0, q] and z, a, b in [0, 27].  In that range 8-bit wrapping
 * add/sub, unsigned max/min and signed compares give the same results as plain
 * int32 arithmetic.  This program runs the per-cell recurrence both ways (the
 * SSE2 byte sequence and the int32 form) over random segments - uniform,
 * similar, N-rich and low-complexity - and counts any difference in the
 * direction byte or the carried state.  Exit code 0 = identical.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

static uint64_t rs = 88172645463325252ull;
static uint32_t rnd(void)
{
    rs ^= rs << 13, rs ^= rs >> 7, rs ^= rs << 17;
    return (uint32_t)(rs >> 11);
}
static inline int8_t s8(uint32_t v) { return (int8_t)(uint8_t)v; }

typedef struct { uint32_t u, v, x, y, d; } lane_t;

static lane_t lane_bytes(uint32_t s, uint32_t xt1, uint32_t vt1, uint32_t ut, uint32_t yt, int mode)
{
    const uint32_t qe2 = 16, max_sc = 21, q = 6;
    uint32_t z = (s + qe2) & 0xff, a = (xt1 + vt1) & 0xff, b = (yt + ut) & 0xff, d = 0;
    if (mode == 1) {
        d = s8(a) > s8(z) ? 1 : 0;
        z = s8(z) > 0 ? z : 0;
        z = z > a ? z : a;
        if (s8(b) > s8(z)) d = 2;
    } else {
        d = s8(z) > s8(a) ? 0 : 1;
        z = s8(z) > 0 ? z : 0;
        z = z > a ? z : a;
        if (!(s8(z) > s8(b))) d = 2;
    }
    z = z > b ? z : b;
    z = z < max_sc ? z : max_sc;
    lane_t o;
    o.u = (z - vt1) & 0xff, o.v = (z - ut) & 0xff;
    z = (z - q) & 0xff;
    a = (a - z) & 0xff, b = (b - z) & 0xff;
    if (mode == 1) {
        o.x = s8(a) > 0 ? a : 0, o.y = s8(b) > 0 ? b : 0;
        if (s8(a) > 0) d |= 8;
        if (s8(b) > 0) d |= 16;
    } else {
        o.x = s8(a) < 0 ? 0 : a, o.y = s8(b) < 0 ? 0 : b;
        if (!(s8(a) < 0)) d |= 8;
        if (!(s8(b) < 0)) d |= 16;
    }
    o.d = d;
    return o;
}

static lane_t lane_int(int s, int xt1, int vt1, int ut, int yt, int mode)
{
    int z = s + 16, a = xt1 + vt1, b = yt + ut, d;
    if (mode == 1) {
        d = a > z ? 1 : 0;
        z = z > a ? z : a;
        if (b > z) d = 2;
    } else {
        d = z > a ? 0 : 1;
        z = z > a ? z : a;
        if (!(z > b)) d = 2;
    }
    z = z > b ? z : b;
    z = z < 21 ? z : 21;
    lane_t o;
    o.u = (uint32_t)(z - vt1), o.v = (uint32_t)(z - ut);
    z -= 6;
    a -= z, b -= z;
    if (mode == 1) {
        o.x = a > 0 ? a : 0, o.y = b > 0 ? b : 0;
        d |= (a > 0 ? 8 : 0) | (b > 0 ? 16 : 0);
    } else {
        o.x = a < 0 ? 0 : a, o.y = b < 0 ? 0 : b;
        d |= (a < 0 ? 0 : 8) | (b < 0 ? 0 : 16);
    }
    o.d = (uint32_t)d;
    return o;
}

static int score(int a, int b) { return (a == 4 || b == 4) ? 0 : (a == b ? 5 : -4); }

int main(int argc, char** argv)
{
    const long trials = argc > 1 ? atol(argv[1]) : 200000;
    long cells = 0, bad = 0;
    int qs[256], ts[256];
    uint32_t U[256], Y[256];
    for (long it = 0; it < trials; ++it) {
        const int qn = 1 + rnd() % 200, tn = 1 + rnd() % 200, kind = rnd() % 5;
        for (int i = 0; i < qn; ++i) qs[i] = rnd() % 4;
        for (int i = 0; i < tn; ++i) {
            if (kind == 1) ts[i] = i < qn && rnd() % 10 ? qs[i] : rnd() % 4;      /* similar */
            else if (kind == 2) ts[i] = rnd() % 3 ? 4 : rnd() % 4;               /* N-rich */
            else if (kind == 3) ts[i] = (i / (1 + rnd() % 3)) & 1;                /* low complexity */
            else ts[i] = rnd() % 5;                                               /* uniform with N */
        }
        if (kind == 2)
            for (int i = 0; i < qn; ++i) qs[i] = rnd() % 2 ? 4 : qs[i];
        const int mode = 1 + rnd() % 2;
        for (int j = 0; j < qn; ++j) {
            uint32_t xb = 0, vb = j ? 6 : 0;
            int xi = 0, vi = j ? 6 : 0;
            for (int t = 0; t < tn; ++t) {
                const uint32_t ut = j ? U[t] : (t ? 6 : 0), yt = j ? Y[t] : 0;
                const int s = score(ts[t], qs[j]);
                const lane_t A = lane_bytes((uint32_t)s & 0xff, xb, vb, ut, yt, mode);
                const lane_t B = lane_int(s, xi, vi, (int)ut, (int)yt, mode);
                if (A.d != B.d || A.u != B.u || A.v != B.v || A.x != B.x || A.y != B.y) ++bad;
                U[t] = A.u, Y[t] = A.y, xb = A.x, vb = A.v;
                xi = (int)B.x, vi = (int)B.v;
                ++cells;
            }
        }
    }
    printf("cells=%ld mismatches=%ld\n", cells, bad);
    return bad != 0;
}
