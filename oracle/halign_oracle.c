/* halign_oracle.c - CPU restatement of HAlign-4's align-to-center path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  Only tests/, the smoke check and
 * bench.py's CPU-baseline leg load this library; the product never does.
 *
 * Each function restates one reference function (file:line cited at the
 * function).  Parity pin: tests/test_oracle_pin.py runs every function here
 * against the unmodified reference sources compiled by oracle/build.py, and
 * tests/test_golden.py replays golden vectors that the reference produced.
 */
#include "halign_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#define KSW_NEG_INF (-0x40000000)
#define EZ_SCORE_ONLY 0x01
#define EZ_RIGHT 0x02
#define EZ_GENERIC_SC 0x04
#define EZ_APPROX_MAX 0x08
#define EZ_APPROX_DROP 0x10
#define EZ_EXTZ_ONLY 0x40
#define EZ_REV_CIGAR 0x80

/* ------------------------------------------------------------------ tables */

/* log2f(i) bit patterns for i = 0..512 as the reference host's libm returns
 * them (mg_log2 returns 0 below 1); src/seed/anchor.cpp:227-230. */
static const uint32_t k_log2_bits[513] = {
    0x00000000u, 0x00000000u, 0x3f800000u, 0x3fcae00du, 0x40000000u, 0x40149a78u, 0x40257007u, 0x4033abb4u,
    0x40400000u, 0x404ae00du, 0x40549a78u, 0x405d6754u, 0x40657007u, 0x406cd401u, 0x4073abb4u, 0x407a0a7fu,
    0x40800000u, 0x4082cc7fu, 0x40857007u, 0x4087ef06u, 0x408a4d3cu, 0x408c8dddu, 0x408eb3aau, 0x4090c105u,
    0x4092b803u, 0x40949a78u, 0x40966a01u, 0x4098280au, 0x4099d5dau, 0x409b7495u, 0x409d053fu, 0x409e88c7u,
    0x40a00000u, 0x40a16badu, 0x40a2cc7fu, 0x40a42316u, 0x40a57007u, 0x40a6b3d8u, 0x40a7ef06u, 0x40a92204u,
    0x40aa4d3cu, 0x40ab7111u, 0x40ac8dddu, 0x40ada3f6u, 0x40aeb3aau, 0x40afbd43u, 0x40b0c105u, 0x40b1bf31u,
    0x40b2b803u, 0x40b3abb4u, 0x40b49a78u, 0x40b58482u, 0x40b66a01u, 0x40b74b20u, 0x40b8280au, 0x40b900e6u,
    0x40b9d5dau, 0x40baa709u, 0x40bb7495u, 0x40bc3e9du, 0x40bd053fu, 0x40bdc89au, 0x40be88c7u, 0x40bf45e1u,
    0x40c00000u, 0x40c0b73du, 0x40c16badu, 0x40c21d67u, 0x40c2cc7fu, 0x40c37908u, 0x40c42316u, 0x40c4cabau,
    0x40c57007u, 0x40c6130bu, 0x40c6b3d8u, 0x40c7527cu, 0x40c7ef06u, 0x40c88984u, 0x40c92204u, 0x40c9b892u,
    0x40ca4d3cu, 0x40cae00du, 0x40cb7111u, 0x40cc0053u, 0x40cc8dddu, 0x40cd19bbu, 0x40cda3f6u, 0x40ce2c98u,
    0x40ceb3aau, 0x40cf3935u, 0x40cfbd43u, 0x40d03fdbu, 0x40d0c105u, 0x40d140cau, 0x40d1bf31u, 0x40d23c42u,
    0x40d2b803u, 0x40d3327cu, 0x40d3abb4u, 0x40d423b0u, 0x40d49a78u, 0x40d51012u, 0x40d58482u, 0x40d5f7d0u,
    0x40d66a01u, 0x40d6db19u, 0x40d74b20u, 0x40d7ba19u, 0x40d8280au, 0x40d894f7u, 0x40d900e6u, 0x40d96bdbu,
    0x40d9d5dau, 0x40da3ee8u, 0x40daa709u, 0x40db0e41u, 0x40db7495u, 0x40dbda07u, 0x40dc3e9du, 0x40dca259u,
    0x40dd053fu, 0x40dd6754u, 0x40ddc89au, 0x40de2914u, 0x40de88c7u, 0x40dee7b4u, 0x40df45e1u, 0x40dfa34eu,
    0x40e00000u, 0x40e05bf9u, 0x40e0b73du, 0x40e111cdu, 0x40e16badu, 0x40e1c4e0u, 0x40e21d67u, 0x40e27546u,
    0x40e2cc7fu, 0x40e32314u, 0x40e37908u, 0x40e3ce5eu, 0x40e42316u, 0x40e47734u, 0x40e4cabau, 0x40e51daau,
    0x40e57007u, 0x40e5c1d1u, 0x40e6130bu, 0x40e663b7u, 0x40e6b3d8u, 0x40e7036eu, 0x40e7527cu, 0x40e7a103u,
    0x40e7ef06u, 0x40e83c85u, 0x40e88984u, 0x40e8d603u, 0x40e92204u, 0x40e96d88u, 0x40e9b892u, 0x40ea0323u,
    0x40ea4d3cu, 0x40ea96dfu, 0x40eae00du, 0x40eb28c8u, 0x40eb7111u, 0x40ebb8e9u, 0x40ec0053u, 0x40ec474eu,
    0x40ec8dddu, 0x40ecd401u, 0x40ed19bbu, 0x40ed5f0cu, 0x40eda3f6u, 0x40ede879u, 0x40ee2c98u, 0x40ee7052u,
    0x40eeb3aau, 0x40eef6a0u, 0x40ef3935u, 0x40ef7b6bu, 0x40efbd43u, 0x40effebdu, 0x40f03fdbu, 0x40f0809du,
    0x40f0c105u, 0x40f10114u, 0x40f140cau, 0x40f18029u, 0x40f1bf31u, 0x40f1fde4u, 0x40f23c42u, 0x40f27a4cu,
    0x40f2b803u, 0x40f2f568u, 0x40f3327cu, 0x40f36f40u, 0x40f3abb4u, 0x40f3e7d9u, 0x40f423b0u, 0x40f45f3bu,
    0x40f49a78u, 0x40f4d56au, 0x40f51012u, 0x40f54a6fu, 0x40f58482u, 0x40f5be4du, 0x40f5f7d0u, 0x40f6310cu,
    0x40f66a01u, 0x40f6a2b0u, 0x40f6db19u, 0x40f7133fu, 0x40f74b20u, 0x40f782beu, 0x40f7ba19u, 0x40f7f132u,
    0x40f8280au, 0x40f85ea1u, 0x40f894f7u, 0x40f8cb0eu, 0x40f900e6u, 0x40f9367fu, 0x40f96bdbu, 0x40f9a0f9u,
    0x40f9d5dau, 0x40fa0a7fu, 0x40fa3ee8u, 0x40fa7316u, 0x40faa709u, 0x40fadac2u, 0x40fb0e41u, 0x40fb4187u,
    0x40fb7495u, 0x40fba76au, 0x40fbda07u, 0x40fc0c6du, 0x40fc3e9du, 0x40fc7096u, 0x40fca259u, 0x40fcd3e7u,
    0x40fd053fu, 0x40fd3664u, 0x40fd6754u, 0x40fd9810u, 0x40fdc89au, 0x40fdf8f0u, 0x40fe2914u, 0x40fe5906u,
    0x40fe88c7u, 0x40feb856u, 0x40fee7b4u, 0x40ff16e3u, 0x40ff45e1u, 0x40ff74afu, 0x40ffa34eu, 0x40ffd1beu,
    0x41000000u, 0x4100170au, 0x41002dfdu, 0x410044d9u, 0x41005b9eu, 0x4100724eu, 0x410088e7u, 0x41009f6au,
    0x4100b5d7u, 0x4100cc2eu, 0x4100e270u, 0x4100f89cu, 0x41010eb4u, 0x410124b6u, 0x41013aa3u, 0x4101507cu,
    0x4101663fu, 0x41017befu, 0x4101918au, 0x4101a711u, 0x4101bc84u, 0x4101d1e3u, 0x4101e72fu, 0x4101fc67u,
    0x4102118bu, 0x4102269cu, 0x41023b9au, 0x41025085u, 0x4102655du, 0x41027a23u, 0x41028ed5u, 0x4102a375u,
    0x4102b803u, 0x4102cc7fu, 0x4102e0e8u, 0x4102f540u, 0x41030985u, 0x41031db9u, 0x410331dcu, 0x410345ecu,
    0x410359ecu, 0x41036ddau, 0x410381b7u, 0x41039583u, 0x4103a93eu, 0x4103bce8u, 0x4103d081u, 0x4103e40au,
    0x4103f783u, 0x41040aebu, 0x41041e43u, 0x4104318au, 0x410444c2u, 0x410457eau, 0x41046b01u, 0x41047e09u,
    0x41049102u, 0x4104a3ebu, 0x4104b6c4u, 0x4104c98eu, 0x4104dc49u, 0x4104eef5u, 0x41050192u, 0x4105141fu,
    0x4105269eu, 0x4105390eu, 0x41054b6fu, 0x41055dc2u, 0x41057007u, 0x4105823cu, 0x41059464u, 0x4105a67du,
    0x4105b888u, 0x4105ca86u, 0x4105dc75u, 0x4105ee56u, 0x41060029u, 0x410611efu, 0x410623a7u, 0x41063552u,
    0x410646efu, 0x4106587eu, 0x41066a01u, 0x41067b76u, 0x41068cdeu, 0x41069e38u, 0x4106af86u, 0x4106c0c7u,
    0x4106d1fbu, 0x4106e322u, 0x4106f43du, 0x4107054bu, 0x4107164cu, 0x41072741u, 0x41073829u, 0x41074905u,
    0x410759d5u, 0x41076a99u, 0x41077b50u, 0x41078bfbu, 0x41079c9bu, 0x4107ad2eu, 0x4107bdb6u, 0x4107ce31u,
    0x4107dea1u, 0x4107ef06u, 0x4107ff5eu, 0x41080facu, 0x41081fedu, 0x41083024u, 0x4108404eu, 0x4108506eu,
    0x41086083u, 0x4108708cu, 0x4108808au, 0x4108907du, 0x4108a065u, 0x4108b042u, 0x4108c014u, 0x4108cfdcu,
    0x4108df99u, 0x4108ef4bu, 0x4108fef2u, 0x41090e8fu, 0x41091e21u, 0x41092da9u, 0x41093d26u, 0x41094c99u,
    0x41095c02u, 0x41096b60u, 0x41097ab4u, 0x410989feu, 0x4109993eu, 0x4109a874u, 0x4109b7a0u, 0x4109c6c2u,
    0x4109d5dau, 0x4109e4e8u, 0x4109f3edu, 0x410a02e7u, 0x410a11d8u, 0x410a20c0u, 0x410a2f9du, 0x410a3e71u,
    0x410a4d3cu, 0x410a5bfdu, 0x410a6ab5u, 0x410a7964u, 0x410a8809u, 0x410a96a5u, 0x410aa537u, 0x410ab3c1u,
    0x410ac241u, 0x410ad0b8u, 0x410adf27u, 0x410aed8cu, 0x410afbe8u, 0x410b0a3bu, 0x410b1886u, 0x410b26c7u,
    0x410b3500u, 0x410b4330u, 0x410b5158u, 0x410b5f77u, 0x410b6d8du, 0x410b7b9au, 0x410b899fu, 0x410b979cu,
    0x410ba590u, 0x410bb37cu, 0x410bc15fu, 0x410bcf3au, 0x410bdd0cu, 0x410bead7u, 0x410bf899u, 0x410c0653u,
    0x410c1405u, 0x410c21afu, 0x410c2f50u, 0x410c3ceau, 0x410c4a7cu, 0x410c5805u, 0x410c6587u, 0x410c7301u,
    0x410c8073u, 0x410c8dddu, 0x410c9b40u, 0x410ca89au, 0x410cb5edu, 0x410cc339u, 0x410cd07cu, 0x410cddb8u,
    0x410ceaedu, 0x410cf81au, 0x410d053fu, 0x410d125du, 0x410d1f74u, 0x410d2c83u, 0x410d398bu, 0x410d468bu,
    0x410d5384u, 0x410d6076u, 0x410d6d61u, 0x410d7a44u, 0x410d8721u, 0x410d93f6u, 0x410da0c4u, 0x410dad8au,
    0x410dba4au, 0x410dc703u, 0x410dd3b5u, 0x410de060u, 0x410ded04u, 0x410df9a1u, 0x410e0637u, 0x410e12c6u,
    0x410e1f4eu, 0x410e2bd0u, 0x410e384bu, 0x410e44bfu, 0x410e512cu, 0x410e5d93u, 0x410e69f3u, 0x410e764du,
    0x410e82a0u, 0x410e8eecu, 0x410e9b32u, 0x410ea771u, 0x410eb3aau, 0x410ebfdcu, 0x410ecc08u, 0x410ed82eu,
    0x410ee44du, 0x410ef066u, 0x410efc78u, 0x410f0884u, 0x410f148au, 0x410f208au, 0x410f2c83u, 0x410f3876u,
    0x410f4463u, 0x410f504au, 0x410f5c2bu, 0x410f6806u, 0x410f73dau, 0x410f7fa9u, 0x410f8b71u, 0x410f9734u,
    0x410fa2f0u, 0x410faea7u, 0x410fba57u, 0x410fc602u, 0x410fd1a7u, 0x410fdd46u, 0x410fe8dfu, 0x410ff472u,
    0x41100000u,
};

const float* ho_log2_table(void) { return (const float*)(const void*)k_log2_bits; }

/* nt4_table (include/seed.h:157-190): ACGT/acgt -> 0..3, U/u -> 3, else 4. */
static uint8_t nt4(unsigned char c)
{
    switch (c) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': case 'U': case 'u': return 3;
    default: return 4;
    }
}

/* ScoreChar2Idx (include/align.h:72-89): ACGT/acgt -> 0..3, else 4 (U too). */
static uint8_t dna5(unsigned char c)
{
    switch (c) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
    default: return 4;
    }
}

/* dna5_simd_mat (include/align.h:109-116). */
static const int8_t k_dna5_mat[25] = {5, -4, -4, -4, 0, -4, 5, -4, -4, 0, -4, -4, 5, -4, 0,
                                      -4, -4, -4, 5, 0, 0,  0,  0,  0,  0};

void ho_default_chain_params(ho_chain_params* p)
{
    p->max_dist_x = 5000;
    p->max_dist_y = 5000;
    p->bw = 500;
    p->max_skip = 25;
    p->max_iter = 5000;
    p->min_cnt = 3;
    p->min_score = 40;
    p->gap_penalty = 0.01f;
    p->skip_penalty = 0.01f;
}

void ho_default_filter_params(ho_filter_params* p)
{
    p->f_top_frac = 2e-4;
    p->u_floor = 10;
    p->u_ceil = 1000000;
    p->q_occ_frac = 0.01;
    p->sample_every_bp = 500;
}

/* ------------------------------------------------------------- A1 minimizer */

static inline uint64_t splitmix64(uint64_t x)
{ /* src/seed/minimizer.cpp:16-22 */
    x += 0x9e3779b97f4a7c15ULL;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
    return x ^ (x >> 31);
}

/* Follows extractMinimizer (src/seed/minimizer.cpp:103-177): rolling 2-bit
 * k-mer, window-minimum deque where a new entry evicts every back entry with
 * hash >= its own (the latest equal hash wins), an invalid base clears the
 * k-mer, the deque and the last-emitted memory, and a minimizer is emitted
 * whenever (hash,pos) differs from the last one emitted. */
static _Thread_local int64_t g_ring_oob = 0;

/* Slot indices >= win used by the last ho_extract_minimizer call on this
 * thread (the reference writes past its buffer there: undefined behaviour). */
int64_t ho_last_ring_oob(void) { return g_ring_oob; }

int64_t ho_extract_minimizer(const char* seq, int64_t n64, int k, int w, int non_canonical,
                             uint64_t* xs, uint64_t* ys, int64_t cap)
{
    g_ring_oob = 0;
    const uint32_t n = (uint32_t)n64;
    if (k == 0 || w == 0 || n < (uint32_t)k) return 0;
    if (k > 31) return 0;
    if (w >= 256) return 0;
    const uint32_t total = n - (uint32_t)k + 1;
    const uint32_t win = (uint32_t)w < total ? (uint32_t)w : total;
    if (win == 0) return 0;
    const uint64_t mask = (1ULL << (2 * k)) - 1ULL;
    const uint64_t shift = 2ULL * (uint64_t)(k - 1);
    uint64_t fwd = 0, rev = 0;
    uint32_t valid = 0;
    /* Deque as a ring of capacity win with the reference's index rule
     * (RingMinQueue::idx subtracts the capacity once).  A push happens before
     * expiry, so after win+1 strictly increasing hashes the deque holds win+1
     * entries and the new entry lands on the front slot; the reference keeps
     * going from that state, and so does this restatement.  Indices past the
     * capacity (reachable only after several such pushes in a row) address
     * spare slots here, i.e. they behave as plain memory. */
    const uint32_t slots = 2 * win + 16;
    uint64_t* qh = (uint64_t*)calloc(slots, sizeof(uint64_t));
    uint32_t* qp = (uint32_t*)calloc(slots, sizeof(uint32_t));
    uint32_t head = 0, size = 0;
    uint64_t last_h = 0;
    uint32_t last_p = 0;
    int has_last = 0;
    int64_t m = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const uint8_t c = nt4((unsigned char)seq[i]);
        if (c >= 4) {
            fwd = rev = 0;
            valid = 0;
            head = size = 0;
            has_last = 0;
            continue;
        }
        fwd = ((fwd << 2) | c) & mask;
        rev = (rev >> 2) | ((uint64_t)(3U ^ c) << shift);
        if (valid < (uint32_t)k) ++valid;
        if (valid < (uint32_t)k) continue;
        const uint32_t pos = i + 1 - (uint32_t)k;
        const uint64_t code = non_canonical ? fwd : (fwd < rev ? fwd : rev);
        const uint64_t h56 = splitmix64(code) >> 8;
        while (size) {
            uint32_t bi = head + size - 1;
            if (bi >= win) bi -= win;
            if (bi >= win) ++g_ring_oob;
            if (qh[bi] >= h56) --size;
            else break;
        }
        {
            uint32_t bi = head + size;
            if (bi >= win) bi -= win;
            if (bi >= win) ++g_ring_oob;
            if (bi >= slots) bi = slots - 1; /* never reached in practice */
            qh[bi] = h56;
            qp[bi] = pos;
            ++size;
        }
        if (pos + 1 < win) continue;
        const uint32_t win_start = pos + 1 - win;
        while (size && qp[head] < win_start) {
            head = head + 1 == win ? 0 : head + 1;
            --size;
        }
        if (size) {
            const uint64_t ch = qh[head];
            const uint32_t cp = qp[head];
            if (!has_last || ch != last_h || cp != last_p) {
                const int strand = non_canonical ? 1 : (fwd <= rev);
                if (m < cap) {
                    xs[m] = (ch << 8) | (uint64_t)(uint8_t)k;
                    ys[m] = ((uint64_t)(strand ? 0x80000000U : 0U) << 32) | (uint64_t)cp;
                }
                ++m;
                last_h = ch;
                last_p = cp;
                has_last = 1;
            }
        }
    }
    free(qh);
    free(qp);
    return m <= cap ? m : -m;
}

/* --------------------------------------------------------------- A2 anchors */

typedef struct {
    uint64_t x, y;
} hit_t;

static inline uint64_t hit_hash(const hit_t* h) { return h->x >> 8; }
static inline uint32_t hit_pos(const hit_t* h) { return (uint32_t)h->y; }
static inline uint32_t hit_rid(const hit_t* h) { return (uint32_t)(h->y >> 32) & 0x7fffffffU; }
static inline uint32_t hit_strand(const hit_t* h) { return (uint32_t)(h->y >> 63); }
static inline uint32_t hit_span(const hit_t* h) { return (uint32_t)(h->x & 0xff); }

/* SeedHitBase::operator< (include/seed.h:68-74): hash, rid, pos, strand. */
static int hit_less(const hit_t* a, const hit_t* b)
{
    if (hit_hash(a) != hit_hash(b)) return hit_hash(a) < hit_hash(b);
    if (hit_rid(a) != hit_rid(b)) return hit_rid(a) < hit_rid(b);
    if (hit_pos(a) != hit_pos(b)) return hit_pos(a) < hit_pos(b);
    return hit_strand(a) < hit_strand(b);
}

static void hit_merge_sort(hit_t* a, hit_t* tmp, int64_t n)
{
    if (n < 2) return;
    if (n <= 16) { /* insertion sort below 16 elements: stable as the merge */
        for (int64_t i = 1; i < n; ++i) {
            const hit_t k = a[i];
            int64_t j = i - 1;
            while (j >= 0 && hit_less(&k, &a[j])) a[j + 1] = a[j], --j;
            a[j + 1] = k;
        }
        return;
    }
    const int64_t h = n / 2;
    hit_merge_sort(a, tmp, h);
    hit_merge_sort(a + h, tmp, n - h);
    int64_t i = 0, j = h, o = 0;
    while (i < h && j < n) tmp[o++] = hit_less(&a[j], &a[i]) ? a[j++] : a[i++];
    while (i < h) tmp[o++] = a[i++];
    while (j < n) tmp[o++] = a[j++];
    memcpy(a, tmp, sizeof(hit_t) * (size_t)n);
}

static int cmp_u64_desc(const void* a, const void* b)
{
    const uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? 1 : (x > y ? -1 : 0);
}

/* compute_ref_occ_threshold / compute_occ_cutoff_top_frac
 * (src/seed/anchor.cpp:73-117). */
uint64_t ho_ref_occ_threshold(const uint64_t* occs, int64_t n, const ho_filter_params* p)
{
    uint64_t f_cut;
    if (n == 0 || p->f_top_frac <= 0.0) f_cut = UINT64_MAX;
    else if (p->f_top_frac >= 1.0) f_cut = 1;
    else {
        const uint64_t n_skip = (uint64_t)floor(p->f_top_frac * (double)n);
        if (n_skip == 0) f_cut = UINT64_MAX;
        else {
            uint64_t* t = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)n);
            memcpy(t, occs, sizeof(uint64_t) * (size_t)n);
            qsort(t, (size_t)n, sizeof(uint64_t), cmp_u64_desc);
            f_cut = t[n_skip - 1];
            free(t);
        }
    }
    const uint64_t capped = p->u_ceil < f_cut ? p->u_ceil : f_cut;
    return p->u_floor > capped ? p->u_floor : capped;
}

/* Binary search for the first sorted hit with the given hash. */
static int64_t lower_bound_hash(const hit_t* s, int64_t n, uint64_t h)
{
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = (lo + hi) / 2;
        if (hit_hash(&s[mid]) < h) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

/* Follows collect_anchors (src/seed/minimizer.cpp:220-356): sort the ref hits,
 * derive the occurrence threshold over distinct hashes, drop query hashes
 * whose query-side count exceeds q_occ_frac * |query hits|, sample
 * over-threshold ref hashes at query positions divisible by sample_every_bp,
 * and expand each surviving query hit over its ref occurrences in sorted
 * order.  (The reference keys a hash map; binary search over the sorted hits
 * finds the same (start, count) ranges.) */
int64_t ho_collect_anchors(const uint64_t* rx, const uint64_t* ry, int64_t nr,
                           const uint64_t* qx, const uint64_t* qy, int64_t nq,
                           const ho_filter_params* fp_in, ho_anchor* out, int64_t cap)
{
    if (nr == 0 || nq == 0) return 0;
    ho_filter_params fp;
    if (fp_in) fp = *fp_in;
    else ho_default_filter_params(&fp);
    hit_t* s = (hit_t*)malloc(sizeof(hit_t) * (size_t)nr);
    hit_t* tmp = (hit_t*)malloc(sizeof(hit_t) * (size_t)(nr > nq ? nr : nq));
    for (int64_t i = 0; i < nr; ++i) s[i].x = rx[i], s[i].y = ry[i];
    hit_merge_sort(s, tmp, nr);
    uint64_t* occs = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)nr);
    int64_t n_occ = 0, start = 0;
    for (int64_t i = 1; i <= nr; ++i) {
        if (i == nr || hit_hash(&s[i]) != hit_hash(&s[start])) {
            occs[n_occ++] = (uint64_t)(i - start);
            start = i;
        }
    }
    const uint64_t thr = ho_ref_occ_threshold(occs, n_occ, &fp);
    free(occs);
    /* query-side counts: sorted copy of the query hashes */
    uint64_t* qh = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)nq);
    for (int64_t i = 0; i < nq; ++i) qh[i] = qx[i] >> 8;
    {
        hit_t* qs = tmp;
        for (int64_t i = 0; i < nq; ++i) qs[i].x = qh[i] << 8, qs[i].y = 0;
        hit_t* tmp2 = (hit_t*)malloc(sizeof(hit_t) * (size_t)nq);
        hit_merge_sort(qs, tmp2, nq);
        free(tmp2);
        for (int64_t i = 0; i < nq; ++i) qh[i] = qs[i].x >> 8; /* sorted hashes */
    }
    const double q_occ_limit = fp.q_occ_frac > 0.0 ? fp.q_occ_frac * (double)nq : INFINITY;
    int64_t m = 0;
    for (int64_t qi = 0; qi < nq; ++qi) {
        hit_t q;
        q.x = qx[qi], q.y = qy[qi];
        const uint64_t h = hit_hash(&q);
        const int64_t lo = lower_bound_hash(s, nr, h);
        if (lo >= nr || hit_hash(&s[lo]) != h) continue;
        int64_t hi = lo;
        while (hi < nr && hit_hash(&s[hi]) == h) ++hi;
        const uint64_t ref_occ = (uint64_t)(hi - lo);
        if (fp.q_occ_frac > 0.0) {
            int64_t a = 0, b = nq;
            while (a < b) {
                const int64_t mid = (a + b) / 2;
                if (qh[mid] < h) a = mid + 1;
                else b = mid;
            }
            int64_t e2 = a;
            while (e2 < nq && qh[e2] == h) ++e2;
            if ((double)(e2 - a) > q_occ_limit) continue;
        }
        if (ref_occ > thr) {
            if (fp.sample_every_bp == 0) continue;
            if ((uint64_t)hit_pos(&q) % fp.sample_every_bp != 0) continue;
        }
        for (int64_t i = lo; i < hi; ++i) {
            if (m < cap) {
                ho_anchor* a = &out[m];
                a->hash = h;
                a->rid_ref = hit_rid(&s[i]);
                a->pos_ref = hit_pos(&s[i]);
                a->rid_qry = hit_rid(&q);
                a->pos_qry = hit_pos(&q);
                a->span = hit_span(&s[i]) < hit_span(&q) ? hit_span(&s[i]) : hit_span(&q);
                a->is_rev = hit_strand(&s[i]) != hit_strand(&q);
            }
            ++m;
        }
    }
    free(qh);
    free(tmp);
    free(s);
    return m <= cap ? m : -m;
}

/* ---------------------------------------------------------- A3/A4 chaining */

static float mg_log2f(float x)
{ /* src/seed/anchor.cpp:227-230, evaluated through the pinned table */
    if (!(x >= 1.0f)) return 0.0f;
    const int i = (int)x;
    if ((float)i == x && i <= 512) return ho_log2_table()[i];
    return log2f(x);
}

/* chainScoreSimple (src/seed/anchor.cpp:254-301). The float penalty is two
 * products and a sum with round-to-nearest after each (no contraction). */
int32_t ho_chain_score(const ho_anchor* ai, const ho_anchor* aj, const ho_chain_params* p)
{
    if (ai->rid_ref != aj->rid_ref) return INT32_MIN;
    if (ai->is_rev != aj->is_rev) return INT32_MIN;
    const int32_t dq = (int32_t)ai->pos_qry - (int32_t)aj->pos_qry;
    if (dq <= 0 || dq > p->max_dist_x) return INT32_MIN;
    const int32_t dr = (int32_t)ai->pos_ref - (int32_t)aj->pos_ref;
    if (dr <= 0 || dr > p->max_dist_y) return INT32_MIN;
    const int32_t dd = dr > dq ? dr - dq : dq - dr;
    if (dd > p->bw) return INT32_MIN;
    const int32_t dg = dr < dq ? dr : dq;
    const int32_t q_span = (int32_t)aj->span;
    int32_t sc = q_span < dg ? q_span : dg;
    if (dd > 0 || dg > q_span) {
        volatile float t1 = p->gap_penalty * (float)dd;
        volatile float t2 = p->skip_penalty * (float)dg;
        volatile float lin = t1 + t2;
        const float lg = dd >= 1 ? mg_log2f((float)(dd + 1)) : 0.0f;
        volatile float half = 0.5f * lg;
        volatile float tot = lin + half;
        sc -= (int32_t)tot;
    }
    return sc;
}

static int anchor_pos_less(const ho_anchor* a, const ho_anchor* b)
{ /* sort key of chainAnchors (src/seed/anchor.cpp:343-349) */
    if (a->rid_ref != b->rid_ref) return a->rid_ref < b->rid_ref;
    if (a->is_rev != b->is_rev) return a->is_rev < b->is_rev;
    if (a->pos_ref != b->pos_ref) return a->pos_ref < b->pos_ref;
    return a->pos_qry < b->pos_qry;
}

static void anchor_merge_sort(ho_anchor* a, ho_anchor* tmp, int64_t n)
{
    if (n < 2) return;
    const int64_t h = n / 2;
    anchor_merge_sort(a, tmp, h);
    anchor_merge_sort(a + h, tmp, n - h);
    int64_t i = 0, j = h, o = 0;
    while (i < h && j < n) tmp[o++] = anchor_pos_less(&a[j], &a[i]) ? a[j++] : a[i++];
    while (i < h) tmp[o++] = a[i++];
    while (j < n) tmp[o++] = a[j++];
    memcpy(a, tmp, sizeof(ho_anchor) * (size_t)n);
}

/* chainAnchors (src/seed/anchor.cpp:332-461): sort, windowed DP with the
 * max_iter cap and the max_skip early exit driven by the t[] marks, global
 * best with strict '>', backtrack, min_score / min_cnt rejection. */
int64_t ho_chain_anchors(ho_anchor* a, int64_t n, const ho_chain_params* p_in, ho_anchor* out, int64_t cap)
{
    return ho_chain_anchors_fp(a, n, p_in, out, cap, 0, 0);
}

int64_t ho_chain_anchors_fp(ho_anchor* a, int64_t n, const ho_chain_params* p_in, ho_anchor* out, int64_t cap,
                            int32_t* f_out, int64_t* p_out)
{
    if (n == 0) return 0;
    ho_chain_params p;
    if (p_in) p = *p_in;
    else ho_default_chain_params(&p);
    ho_anchor* tmp = (ho_anchor*)malloc(sizeof(ho_anchor) * (size_t)n);
    anchor_merge_sort(a, tmp, n);
    free(tmp);
    int32_t* f = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    int64_t* pr = (int64_t*)calloc((size_t)n, sizeof(int64_t));
    int32_t* t = (int32_t*)calloc((size_t)n, sizeof(int32_t));
    int64_t st = 0, best = -1;
    int32_t best_f = 0;
    for (int64_t i = 0; i < n; ++i) {
        const ho_anchor* ai = &a[i];
        int32_t max_f = (int32_t)ai->span;
        int64_t max_j = -1;
        int32_t n_skip = 0;
        while (st < i) {
            const ho_anchor* s = &a[st];
            if (s->rid_ref != ai->rid_ref || s->is_rev != ai->is_rev ||
                (int32_t)(ai->pos_ref - s->pos_ref) > p.max_dist_x)
                ++st;
            else
                break;
        }
        const int64_t it0 = (i - st > p.max_iter) ? (i - p.max_iter) : st;
        for (int64_t j = i - 1; j >= it0; --j) {
            const int32_t sc = ho_chain_score(ai, &a[j], &p);
            if (sc == INT32_MIN) continue;
            const int32_t tot = f[j] + sc;
            if (tot > max_f) {
                max_f = tot;
                max_j = j;
                if (n_skip > 0) --n_skip;
            } else if (t[j] == (int32_t)i) {
                if (++n_skip > p.max_skip) break;
            }
            if (pr[j] >= 0) t[pr[j]] = (int32_t)i;
        }
        f[i] = max_f;
        pr[i] = max_j;
        if (max_f > best_f) best_f = max_f, best = i;
    }
    if (f_out) memcpy(f_out, f, sizeof(int32_t) * (size_t)n);
    if (p_out) memcpy(p_out, pr, sizeof(int64_t) * (size_t)n);
    int64_t m = 0;
    if (!(best_f < p.min_score || best < 0)) {
        int64_t len = 0;
        for (int64_t c = best; c >= 0; c = pr[c]) ++len;
        if (len >= p.min_cnt) {
            m = len;
            if (len <= cap) {
                int64_t k = len;
                for (int64_t c = best; c >= 0; c = pr[c]) out[--k] = a[c];
            }
        }
    }
    free(f);
    free(pr);
    free(t);
    return m <= cap ? m : -m;
}

/* -------------------------------------------------------- A7/A8 KSW2 extz2 */

typedef struct {
    uint32_t* v;
    int64_t n, m;
} cig_t;

static void cig_push(cig_t* c, uint32_t op, uint32_t len)
{ /* ksw_push_cigar (include/ksw2.h:113-123) */
    if (c->n == 0 || op != (c->v[c->n - 1] & 0xf)) {
        if (c->n == c->m) {
            c->m = c->m ? c->m << 1 : 4;
            c->v = (uint32_t*)realloc(c->v, sizeof(uint32_t) * (size_t)c->m);
        }
        c->v[c->n++] = len << 4 | op;
    } else
        c->v[c->n - 1] += len << 4;
}

/* ksw_backtrack (include/ksw2.h:129-161), rotated (anti-diagonal) layout,
 * no introns. */
static void backtrack(int is_rev, const uint8_t* p, const int* off, const int* off_end, size_t n_col, int i0,
                      int j0, cig_t* c)
{
    int i = i0, j = j0, state = 0;
    while (i >= 0 && j >= 0) {
        const int r = i + j;
        int force = -1;
        uint32_t tmp;
        if (i < off[r]) force = 2;
        if (i > off_end[r]) force = 1;
        tmp = force < 0 ? p[(size_t)r * n_col + (size_t)(i - off[r])] : 0;
        if (state == 0) state = tmp & 7;
        else if (!(tmp >> (state + 2) & 1)) state = 0;
        if (state == 0) state = tmp & 7;
        if (force >= 0) state = force;
        if (state == 0) cig_push(c, 0, 1), --i, --j;
        else if (state == 1 || state == 3) cig_push(c, 2, 1), --i;
        else cig_push(c, 1, 1), --j;
    }
    if (i >= 0) cig_push(c, 2, (uint32_t)(i + 1));
    if (j >= 0) cig_push(c, 1, (uint32_t)(j + 1));
    if (!is_rev)
        for (int64_t k = 0; k < c->n >> 1; ++k) {
            const uint32_t t = c->v[k];
            c->v[k] = c->v[c->n - 1 - k];
            c->v[c->n - 1 - k] = t;
        }
}

static int apply_zdrop(ho_extz* ez, int32_t H, int r, int t, int zdrop, int8_t e)
{ /* ksw_apply_zdrop (include/ksw2.h:191-207), rotated coordinates */
    if (H > ez->max) {
        ez->max = H, ez->max_t = t, ez->max_q = r - t;
    } else if (t >= ez->max_t && r - t >= ez->max_q) {
        const int tl = t - ez->max_t, ql = (r - t) - ez->max_q;
        const int l = tl > ql ? tl - ql : ql - tl;
        if (zdrop >= 0 && ez->max - H > zdrop + l * e) {
            ez->zdropped = 1;
            return 1;
        }
    }
    return 0;
}

static inline int8_t s8(uint8_t v) { return (int8_t)v; }

/* 16 byte lanes with GCC vector extensions (SSE2 on x86-64, NEON on
 * aarch64): the SSE2 kernel's operations - wrapping add/sub, unsigned
 * max/min, signed greater-than as an all-ones mask - one block at a time. */
typedef uint8_t u8x16 __attribute__((vector_size(16)));
typedef uint8_t u8x4 __attribute__((vector_size(4)));
typedef int32_t i32x4 __attribute__((vector_size(16)));
typedef int8_t i8x16 __attribute__((vector_size(16)));

static inline u8x16 v16_set(uint8_t c)
{
    const u8x16 zero = {0};
    return zero + c; /* the scalar is broadcast to every lane */
}
static inline u8x16 v16_load(const uint8_t* p)
{
    u8x16 r;
    memcpy(&r, p, 16);
    return r;
}
static inline void v16_store(uint8_t* p, u8x16 v) { memcpy(p, &v, 16); }
static inline u8x16 v16_gts(u8x16 a, u8x16 b) { return (u8x16)((i8x16)a > (i8x16)b); }
static inline u8x16 v16_sel(u8x16 m, u8x16 a, u8x16 b) { return (m & a) | (~m & b); }
static inline u8x16 v16_maxu(u8x16 a, u8x16 b) { return v16_sel((u8x16)(a > b), a, b); }
static inline u8x16 v16_minu(u8x16 a, u8x16 b) { return v16_sel((u8x16)(a < b), a, b); }
/* lane i <- lane i-1, lane 0 <- 0 */
static inline u8x16 v16_shift_in(u8x16 a)
{
    const u8x16 zero = {0};
    const u8x16 idx = {16, 0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14};
    return __builtin_shuffle(a, zero, idx);
}

/* ksw_extz2_sse (src/align/ksw2_extz2_sse.c:23-304) as compiled for plain
 * SSE2, restated one byte lane at a time.  The anti-diagonal sweep keeps the
 * reference's per-target-position byte arrays u, v, x, y, s and its rounding
 * of every band row to whole 16-lane blocks, so lanes outside [st0, en0] are
 * computed (from stale s[] and state) exactly as the SIMD code does.  Each
 * lane applies the SSE2 instruction sequence: 8-bit wrapping add/sub,
 * unsigned max/min, signed compares. */
int64_t ho_ksw_extz2(int qlen, const uint8_t* query, int tlen, const uint8_t* target, int8_t m,
                     const int8_t* mat, int8_t q, int8_t e, int w, int zdrop, int end_bonus, int flag,
                     ho_extz* ez, uint32_t* cigar_out, int64_t cap)
{
    const int qe = q + e, with_cigar = !(flag & EZ_SCORE_ONLY), approx_max = !!(flag & EZ_APPROX_MAX);
    ez->max_q = ez->max_t = ez->mqe_t = ez->mte_q = -1;
    ez->max = 0, ez->score = ez->mqe = ez->mte = KSW_NEG_INF;
    ez->zdropped = 0, ez->reach_end = 0;
    if (m <= 0 || qlen <= 0 || tlen <= 0) return 0;
    const uint8_t qe2 = (uint8_t)((q + e) * 2);
    const uint8_t max_sc = (uint8_t)(mat[0] + (q + e) * 2);
    if (w < 0) w = tlen > qlen ? tlen : qlen;
    const int wl = w, wr = w;
    const int tlen_ = (tlen + 15) / 16;
    int n_col_ = qlen < tlen ? qlen : tlen;
    n_col_ = ((n_col_ < w + 1 ? n_col_ : w + 1) + 15) / 16 + 1;
    int min_sc = mat[1];
    for (int t = 1; t < m * m; ++t) min_sc = min_sc < mat[t] ? min_sc : mat[t];
    if (-min_sc > 2 * (q + e)) return 0;

    const size_t L = (size_t)tlen_ * 16;
    /* one block: u v x y s (L bytes each), H (L int32), off/off_end, p */
    const size_t ncol = (size_t)n_col_ * 16;
    const size_t nd = (size_t)(qlen + tlen - 1);
    const size_t p_bytes = with_cigar ? (nd * (size_t)n_col_ + 1) * 16 : 0;
    uint8_t* blk = (uint8_t*)malloc(L * 5 + sizeof(int32_t) * L + (with_cigar ? sizeof(int) * nd * 2 : 0) + p_bytes);
    uint8_t* u = blk;
    memset(u, 0, L * 5);
    uint8_t *v = u + L, *x = v + L, *y = x + L, *s = y + L;
    int32_t* H = 0;
    int32_t H0 = 0, last_H0_t = 0;
    if (!approx_max) {
        H = (int32_t*)(blk + L * 5);
        for (size_t t = 0; t < L; ++t) H[t] = KSW_NEG_INF;
    }
    uint8_t* p = 0;
    int *off = 0, *off_end = 0;
    if (with_cigar) {
        off = (int*)(blk + L * 5 + sizeof(int32_t) * L);
        off_end = off + nd;
        p = (uint8_t*)(off + 2 * nd);
    }
    int last_st = -1, last_en = -1;
    const int mode = !with_cigar ? 0 : !(flag & EZ_RIGHT) ? 1 : 2;
    const u8x16 k0 = v16_set(0), kqe2 = v16_set(qe2), kq = v16_set((uint8_t)q), kmax = v16_set(max_sc);
    const u8x16 k1 = v16_set(1), k2 = v16_set(2), k8 = v16_set(0x08), k16 = v16_set(0x10);
    const u8x16 m0 = {0xff}, m123 = {0, 0xff, 0xff, 0xff};
    for (int r = 0; r < qlen + tlen - 1; ++r) {
        int st = 0, en = tlen - 1;
        if (st < r - qlen + 1) st = r - qlen + 1;
        if (en > r) en = r;
        if (st < (r - wr + 1) >> 1) st = (r - wr + 1) >> 1;
        if (en > (r + wl) >> 1) en = (r + wl) >> 1;
        if (st > en) {
            ez->zdropped = 1;
            break;
        }
        const int st0 = st, en0 = en;
        st = st / 16 * 16, en = (en + 16) / 16 * 16 - 1;
        uint8_t x1, v1;
        if (st > 0) {
            if (st - 1 >= last_st && st - 1 <= last_en) x1 = x[st - 1], v1 = v[st - 1];
            else x1 = v1 = 0;
        } else
            x1 = 0, v1 = (uint8_t)(r ? q : 0);
        if (en >= r) y[r] = 0, u[r] = (uint8_t)(r ? q : 0);
        if (flag & EZ_GENERIC_SC) {
            for (int t = st0; t <= en0; ++t) s[t] = (uint8_t)mat[target[t] * m + query[r - t]];
        } else {
            /* Match/mismatch scoring, symbol m-1 the wildcard (ksw2_extz2_sse.c:
             * 123-137): 16-byte blocks from st0, so up to 15 lanes past en0 are
             * scored from the reference's buffers - the zero-padded target copy
             * (sf, L bytes) and, past it, the reversed query qr (zeros past
             * qlen).  Lanes at or past L are never computed; not stored. */
            const int scn = mat[m * m - 1] == 0 ? -e : mat[m * m - 1];
            int tend = st0 + ((en0 - st0) / 16 + 1) * 16 - 1;
            if (tend > (int)L - 1) tend = (int)L - 1;
            for (int t = st0; t <= tend; ++t) {
                const int kr = t - (int)L;
                const int sq = t < tlen ? target[t] : t < (int)L ? 0 : (kr < qlen ? query[qlen - 1 - kr] : 0);
                const int kq = qlen - 1 - r + t;
                const int sr = kq < qlen ? query[qlen - 1 - kq] : 0;
                int sc = sq == sr ? mat[0] : mat[1];
                if (sq == m - 1 || sr == m - 1) sc = scn;
                s[t] = (uint8_t)sc;
            }
        }
        uint8_t* pr = with_cigar ? p + (size_t)r * ncol : 0;
        if (with_cigar) off[r] = st, off_end[r] = en;
        /* The SIMD code seeds the first block's shifted-in byte with
         * _mm_cvtsi32_si128(int8): the value is sign-extended into bytes 0-3,
         * so a negative boundary byte ORs 0xFF into lanes st+1..st+3. */
        const uint8_t x1_ext = s8(x1) < 0 ? 0xff : 0, v1_ext = s8(v1) < 0 ? 0xff : 0;
        /* 16 lanes per step, as the SSE2 code (st and en + 1 are multiples of
         * 16): lane i of a block reads lane i-1 of the previous anti-diagonal,
         * lane 0 the carried byte of the block before. */
        for (int t = st; t <= en; t += 16) {
            /* carried byte in lane 0 (and, in the first block, the sign
             * extension in lanes 1-3), built with masks: element insertion
             * would go through memory */
            u8x16 cx = v16_set(x1) & m0, cv = v16_set(v1) & m0;
            if (t == st) cx |= v16_set(x1_ext) & m123, cv |= v16_set(v1_ext) & m123;
            const u8x16 X = v16_load(x + t), Vv = v16_load(v + t), ut = v16_load(u + t), yt = v16_load(y + t);
            x1 = x[t + 15], v1 = v[t + 15];
            const u8x16 xt1 = v16_shift_in(X) | cx, vt1 = v16_shift_in(Vv) | cv;
            u8x16 z = v16_load(s + t) + kqe2;
            u8x16 a = xt1 + vt1, b = yt + ut, d = k0;
            if (mode == 0) {
                z = v16_sel(v16_gts(z, k0), z, k0);
                z = v16_maxu(z, a);
            } else if (mode == 1) {
                d = v16_gts(a, z) & k1;
                z = v16_sel(v16_gts(z, k0), z, k0);
                z = v16_maxu(z, a);
                d = v16_sel(v16_gts(b, z), k2, d);
            } else {
                d = ~v16_gts(z, a) & k1;
                z = v16_sel(v16_gts(z, k0), z, k0);
                z = v16_maxu(z, a);
                d = v16_sel(v16_gts(z, b), d, k2);
            }
            z = v16_maxu(z, b);
            z = v16_minu(z, kmax);
            v16_store(u + t, z - vt1);
            v16_store(v + t, z - ut);
            z = z - kq;
            a = a - z;
            b = b - z;
            if (mode != 2) {
                const u8x16 pa = v16_gts(a, k0), pb = v16_gts(b, k0);
                v16_store(x + t, a & pa);
                v16_store(y + t, b & pb);
                d |= (pa & k8) | (pb & k16);
            } else {
                const u8x16 na = v16_gts(k0, a), nb = v16_gts(k0, b);
                v16_store(x + t, a & ~na);
                v16_store(y + t, b & ~nb);
                d |= (~na & k8) | (~nb & k16);
            }
            if (with_cigar) v16_store(pr + (t - st), d);
        }
        if (!approx_max) {
            int32_t max_H, max_t;
            if (r > 0) {
                H[en0] = en0 > 0 ? H[en0 - 1] + u[en0] - qe : H[en0] + v[en0] - qe;
                max_H = H[en0], max_t = en0;
                /* four interleaved running maxima (one per 32-bit SIMD lane),
                 * each keeping its first maximum, then combined in lane order */
                const int en1 = st0 + (en0 - st0) / 4 * 4;
                const i32x4 zero4 = {0};
                i32x4 lh = zero4 + max_H, lt = zero4 + max_t;
                const i32x4 kqe = zero4 + qe;
                int t;
                for (t = st0; t < en1; t += 4) {
                    u8x4 vb;
                    memcpy(&vb, v + t, 4);
                    i32x4 h;
                    memcpy(&h, H + t, 16);
                    h += __builtin_convertvector(vb, i32x4) - kqe;
                    memcpy(H + t, &h, 16);
                    const i32x4 gt = h > lh;
                    lh = (gt & h) | (~gt & lh);
                    lt = (gt & (zero4 + t)) | (~gt & lt);
                }
                for (int i = 0; i < 4; ++i)
                    if (max_H < lh[i]) max_H = lh[i], max_t = lt[i] + i;
                for (; t < en0; ++t) {
                    H[t] += (int32_t)v[t] - qe;
                    if (H[t] > max_H) max_H = H[t], max_t = t;
                }
            } else
                H[0] = v[0] - qe - qe, max_H = H[0], max_t = 0;
            if (en0 == tlen - 1 && H[en0] > ez->mte) ez->mte = H[en0], ez->mte_q = r - en;
            if (r - st0 == qlen - 1 && H[st0] > ez->mqe) ez->mqe = H[st0], ez->mqe_t = st0;
            if (apply_zdrop(ez, max_H, r, max_t, zdrop, e)) break;
            if (r == qlen + tlen - 2 && en0 == tlen - 1) ez->score = H[tlen - 1];
        } else {
            if (r > 0) {
                if (last_H0_t >= st0 && last_H0_t <= en0 && last_H0_t + 1 >= st0 && last_H0_t + 1 <= en0) {
                    const int32_t d0 = v[last_H0_t] - qe;
                    const int32_t d1 = u[last_H0_t + 1] - qe;
                    if (d0 > d1) H0 += d0;
                    else H0 += d1, ++last_H0_t;
                } else if (last_H0_t >= st0 && last_H0_t <= en0) {
                    H0 += v[last_H0_t] - qe;
                } else {
                    ++last_H0_t, H0 += u[last_H0_t] - qe;
                }
                if ((flag & EZ_APPROX_DROP) && apply_zdrop(ez, H0, r, last_H0_t, zdrop, e)) break;
            } else
                H0 = v[0] - qe - qe, last_H0_t = 0;
            if (r == qlen + tlen - 2 && en0 == tlen - 1) ez->score = H0;
        }
        last_st = st, last_en = en;
    }
    cig_t c = {0, 0, 0};
    if (with_cigar) {
        const int rev = !!(flag & EZ_REV_CIGAR);
        if (!ez->zdropped && !(flag & EZ_EXTZ_ONLY)) {
            backtrack(rev, p, off, off_end, ncol, tlen - 1, qlen - 1, &c);
        } else if (!ez->zdropped && (flag & EZ_EXTZ_ONLY) && ez->mqe + end_bonus > ez->max) {
            ez->reach_end = 1;
            backtrack(rev, p, off, off_end, ncol, ez->mqe_t, qlen - 1, &c);
        } else if (ez->max_t >= 0 && ez->max_q >= 0) {
            backtrack(rev, p, off, off_end, ncol, ez->max_t, ez->max_q, &c);
        }
    }
    free(blk);
    const int64_t nc = c.n;
    if (nc <= cap && nc) memcpy(cigar_out, c.v, sizeof(uint32_t) * (size_t)nc);
    free(c.v);
    return nc <= cap ? nc : -nc;
}

/* ------------------------------------------------------- A6 globalAlignKSW2 */

int ho_auto_band(int qlen, int tlen)
{ /* include/align.h:159-172 with indel_rate 0.1, margin 200 */
    const int d = qlen - tlen < 0 ? tlen - qlen : qlen - tlen;
    const int mx = qlen > tlen ? qlen : tlen;
    if ((double)d / (double)mx > 0.5) return -1;
    return 200 + (int)(0.1 * (double)(qlen + tlen / 2));
}

static void cig_append(cig_t* res, const uint32_t* add, int64_t n)
{ /* cigar::appendCigar (src/align/cigar.cpp:302-329) */
    for (int64_t i = 0; i < n; ++i) {
        const uint32_t op = add[i] & 0xf, len = add[i] >> 4;
        if (len == 0) continue;
        if (res->n && (res->v[res->n - 1] & 0xf) == op)
            res->v[res->n - 1] = ((( res->v[res->n - 1] >> 4) + len) << 4) | op;
        else {
            if (res->n == res->m) {
                res->m = res->m ? res->m * 2 : 16;
                res->v = (uint32_t*)realloc(res->v, sizeof(uint32_t) * (size_t)res->m);
            }
            res->v[res->n++] = add[i];
        }
    }
}

int64_t ho_cigar_ref_len(const uint32_t* c, int64_t n)
{ /* getRefLength: M D N = X (src/align/cigar.cpp:332-347) */
    int64_t t = 0;
    for (int64_t i = 0; i < n; ++i) {
        const uint32_t op = c[i] & 0xf;
        if (op == 0 || op == 2 || op == 3 || op == 7 || op == 8) t += c[i] >> 4;
    }
    return t;
}

int64_t ho_cigar_query_len(const uint32_t* c, int64_t n)
{ /* getQueryLength: M I S = X (src/align/cigar.cpp:350-365) */
    int64_t t = 0;
    for (int64_t i = 0; i < n; ++i) {
        const uint32_t op = c[i] & 0xf;
        if (op == 0 || op == 1 || op == 4 || op == 7 || op == 8) t += c[i] >> 4;
    }
    return t;
}

int ho_cigar_has_insertion(const uint32_t* c, int64_t n)
{
    for (int64_t i = 0; i < n; ++i)
        if ((c[i] & 0xf) == 1) return 1;
    return 0;
}

/* globalAlignKSW2 (src/align/align.cpp:22-65) into a growable CIGAR. */
static void global_ksw2(const char* ref, int64_t rlen, const char* qry, int64_t qlen, int flag, cig_t* out)
{
    out->n = 0;
    if (rlen == 0 || qlen == 0) {
        if (rlen == 0 && qlen > 0) {
            const uint32_t op = (uint32_t)qlen << 4 | 1;
            cig_append(out, &op, 1);
        } else if (qlen == 0 && rlen > 0) {
            const uint32_t op = (uint32_t)rlen << 4 | 2;
            cig_append(out, &op, 1);
        }
        return;
    }
    /* codes and the CIGAR in one buffer (on the stack for small segments) */
    const int64_t cap = qlen + rlen + 2;
    uint32_t small[256];
    const size_t need = (size_t)cap * 4 + (size_t)rlen + (size_t)qlen;
    uint32_t* c = need <= sizeof(small) ? small : (uint32_t*)malloc(need);
    uint8_t* re = (uint8_t*)(c + cap);
    uint8_t* qe = re + rlen;
    for (int64_t i = 0; i < rlen; ++i) re[i] = dna5((unsigned char)ref[i]);
    for (int64_t i = 0; i < qlen; ++i) qe[i] = dna5((unsigned char)qry[i]);
    const int w = ho_auto_band((int)rlen, (int)qlen);
    ho_extz ez;
    const int64_t nc = ho_ksw_extz2((int)qlen, qe, (int)rlen, re, 5, k_dna5_mat, 6, 2, w, -1, 0,
                                    flag < 0 ? (EZ_GENERIC_SC | EZ_RIGHT) : flag, &ez, c, cap);
    /* the wrapper copies ez.cigar verbatim; no merging */
    for (int64_t i = 0; i < nc; ++i) {
        if (out->n == out->m) {
            out->m = out->m ? out->m * 2 : 16;
            out->v = (uint32_t*)realloc(out->v, sizeof(uint32_t) * (size_t)out->m);
        }
        out->v[out->n++] = c[i];
    }
    if (c != small) free(c);
}

static int64_t emit(const cig_t* c, uint32_t* out, int64_t cap)
{
    if (c->n <= cap && c->n) memcpy(out, c->v, sizeof(uint32_t) * (size_t)c->n);
    return c->n <= cap ? c->n : -c->n;
}

int64_t ho_global_align_ksw2(const char* ref, int64_t rlen, const char* qry, int64_t qlen, int flag,
                             uint32_t* cigar, int64_t cap)
{
    cig_t c = {0, 0, 0};
    global_ksw2(ref, rlen, qry, qlen, flag, &c);
    const int64_t r = emit(&c, cigar, cap);
    free(c.v);
    return r;
}

/* ----------------------------------------------------- A5 globalAlignMM2 */

static int anchor_qry_less(const ho_anchor* a, const ho_anchor* b)
{
    if (a->pos_qry != b->pos_qry) return a->pos_qry < b->pos_qry;
    return a->pos_ref < b->pos_ref;
}

/* globalAlignMM2 (src/align/align.cpp:189-305): chain, sort the chain by
 * (pos_qry, pos_ref), align the left end with left-aligned gaps, then for each
 * anchor the span segment and the gap to the next anchor, then the right end;
 * a segment whose CIGAR does not consume it becomes I(q)D(t); a total that
 * does not cover both sequences falls back to one global alignment. */
static void mm2(const char* ref, int64_t rlen, const char* qry, int64_t qlen, const ho_anchor* anchors,
                int64_t n, cig_t* res)
{
    res->n = 0;
    ho_anchor* sorted = (ho_anchor*)malloc(sizeof(ho_anchor) * (size_t)(n ? n : 1));
    if (n) memcpy(sorted, anchors, sizeof(ho_anchor) * (size_t)n);
    ho_anchor* chain = (ho_anchor*)malloc(sizeof(ho_anchor) * (size_t)(n ? n : 1));
    const int64_t nch = n ? ho_chain_anchors(sorted, n, 0, chain, n) : 0;
    free(sorted);
    if (nch <= 0) {
        free(chain);
        global_ksw2(ref, rlen, qry, qlen, -1, res);
        return;
    }
    /* insertion sort by (pos_qry, pos_ref); the chain is already ordered on
     * this path, so this is linear */
    for (int64_t i = 1; i < nch; ++i) {
        ho_anchor k = chain[i];
        int64_t j = i - 1;
        while (j >= 0 && anchor_qry_less(&k, &chain[j])) chain[j + 1] = chain[j], --j;
        chain[j + 1] = k;
    }
    int64_t ref_pos = 0, qry_pos = 0;
    cig_t seg = {0, 0, 0};
    for (int64_t k = -1; k <= 2 * nch - 1; ++k) {
        int64_t re, qe;
        int flag = -1;
        if (k == -1) { /* left end */
            re = chain[0].pos_ref, qe = chain[0].pos_qry, flag = EZ_GENERIC_SC;
        } else if (k == 2 * nch - 1) { /* right end */
            re = rlen, qe = qlen;
        } else if ((k & 1) == 0) { /* anchor span */
            const ho_anchor* a = &chain[k / 2];
            re = (int64_t)a->pos_ref + a->span, qe = (int64_t)a->pos_qry + a->span;
        } else { /* gap to the next anchor */
            const ho_anchor* b = &chain[k / 2 + 1];
            re = b->pos_ref, qe = b->pos_qry;
        }
        int64_t rs = ref_pos < rlen ? ref_pos : rlen, qs = qry_pos < qlen ? qry_pos : qlen;
        re = re < rlen ? re : rlen;
        qe = qe < qlen ? qe : qlen;
        if (re < rs) re = rs;
        if (qe < qs) qe = qs;
        global_ksw2(ref + rs, re - rs, qry + qs, qe - qs, flag, &seg);
        if (ho_cigar_ref_len(seg.v, seg.n) != re - rs || ho_cigar_query_len(seg.v, seg.n) != qe - qs) {
            uint32_t forced[2];
            int nf = 0;
            if (qe - qs > 0) forced[nf++] = (uint32_t)(qe - qs) << 4 | 1;
            if (re - rs > 0) forced[nf++] = (uint32_t)(re - rs) << 4 | 2;
            cig_append(res, forced, nf);
        } else
            cig_append(res, seg.v, seg.n);
        ref_pos = re;
        qry_pos = qe;
    }
    free(seg.v);
    free(chain);
    if (ho_cigar_ref_len(res->v, res->n) != rlen || ho_cigar_query_len(res->v, res->n) != qlen)
        global_ksw2(ref, rlen, qry, qlen, -1, res);
}

int64_t ho_global_align_mm2(const char* ref, int64_t rlen, const char* qry, int64_t qlen,
                            const ho_anchor* anchors, int64_t n, uint32_t* cigar, int64_t cap)
{
    cig_t c = {0, 0, 0};
    mm2(ref, rlen, qry, qlen, anchors, n, &c);
    const int64_t r = emit(&c, cigar, cap);
    free(c.v);
    return r;
}

/* ------------------------------------------------------- A12 one query */

static int64_t align_query_c(const char* center_dp, int64_t clen, const uint64_t* cmx, const uint64_t* cmy,
                             int64_t ncm, const char* qry, int64_t qlen, int k, int w, cig_t* res)
{
    const int64_t cap = qlen + 1;
    uint64_t* qx = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)cap);
    uint64_t* qy = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)cap);
    const int64_t nq = ho_extract_minimizer(qry, qlen, k, w, 1, qx, qy, cap);
    int64_t acap = nq * 4 + 16, na;
    ho_anchor* an = 0;
    for (;;) {
        an = (ho_anchor*)realloc(an, sizeof(ho_anchor) * (size_t)acap);
        na = ho_collect_anchors(cmx, cmy, ncm, qx, qy, nq, 0, an, acap);
        if (na >= 0) break;
        acap = -na;
    }
    mm2(center_dp, clen, qry, qlen, an, na, res);
    free(an);
    free(qx);
    free(qy);
    return res->n;
}

int64_t ho_align_query(const char* center_dp, int64_t clen, const uint64_t* cmx, const uint64_t* cmy,
                       int64_t ncm, const char* qry, int64_t qlen, int k, int w, uint32_t* cigar, int64_t cap)
{
    cig_t c = {0, 0, 0};
    align_query_c(center_dp, clen, cmx, cmy, ncm, qry, qlen, k, w, &c);
    const int64_t r = emit(&c, cigar, cap);
    free(c.v);
    return r;
}

double ho_align_batch(const char* center_dp, int64_t clen, const char* center_raw, int64_t raw_len,
                      const char* seqs, const int64_t* offsets, int64_t n, int k, int w, int nthreads,
                      uint32_t* cigar, int64_t cap_per_query, int64_t* n_cigar)
{
    const int64_t ccap = raw_len + 1;
    uint64_t* cmx = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)ccap);
    uint64_t* cmy = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)ccap);
    const int64_t ncm = ho_extract_minimizer(center_raw, raw_len, k, w, 1, cmx, cmy, ccap);
    const double t0 = omp_get_wtime();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int64_t i = 0; i < n; ++i) {
        cig_t c = {0, 0, 0};
        align_query_c(center_dp, clen, cmx, cmy, ncm, seqs + offsets[i], offsets[i + 1] - offsets[i], k, w, &c);
        n_cigar[i] = emit(&c, cigar + i * cap_per_query, cap_per_query);
        free(c.v);
    }
    const double dt = omp_get_wtime() - t0;
    free(cmx);
    free(cmy);
    return dt;
}

/* ---------------------------------------------------- A10/A11 rows, counts */

int64_t ho_del_query(const char* qry, int64_t qlen, const uint32_t* c, int64_t n, char* out, int64_t cap)
{ /* delQueryToRefByCigar (src/align/cigar.cpp:212-299): M/S/=/X copy,
   * I skips query bases, D/N write '-', H/P ignored; empty CIGAR = unchanged */
    if (n == 0) {
        if (qlen > cap) return -qlen;
        memcpy(out, qry, (size_t)qlen);
        return qlen;
    }
    int64_t out_len = 0;
    for (int64_t i = 0; i < n; ++i) {
        const uint32_t op = c[i] & 0xf;
        if (op == 1 || op == 5 || op == 6) continue;
        out_len += c[i] >> 4;
    }
    if (out_len > cap) return -out_len;
    int64_t r = 0, o = 0;
    for (int64_t i = 0; i < n; ++i) {
        const uint32_t op = c[i] & 0xf, len = c[i] >> 4;
        if (op == 1) r += len;
        else if (op == 5 || op == 6) continue;
        else if (op == 2 || op == 3) {
            memset(out + o, '-', len);
            o += len;
        } else {
            memcpy(out + o, qry + r, len);
            o += len, r += len;
        }
    }
    return out_len;
}

void ho_count_rows(const char* rows, int64_t n_rows, int64_t L, uint32_t* counts7)
{ /* k_base_map (include/consensus.h:126-145): A C G T U N(default) -/. */
    for (int64_t i = 0; i < n_rows; ++i) {
        const unsigned char* r = (const unsigned char*)rows + i * L;
        for (int64_t c = 0; c < L; ++c) {
            int idx;
            switch (r[c]) {
            case 'A': case 'a': idx = 0; break;
            case 'C': case 'c': idx = 1; break;
            case 'G': case 'g': idx = 2; break;
            case 'T': case 't': idx = 3; break;
            case 'U': case 'u': idx = 4; break;
            case '-': case '.': idx = 6; break;
            default: idx = 5;
            }
            counts7[c * 7 + idx]++;
        }
    }
}

void ho_count_insertions(const uint32_t* c, int64_t n, uint32_t* ins, int64_t L)
{
    int64_t col = 0;
    for (int64_t i = 0; i < n; ++i) {
        const uint32_t op = c[i] & 0xf, len = c[i] >> 4;
        if (op == 1) {
            if (col <= L) ins[col]++;
        } else if (op == 0 || op == 2 || op == 3 || op == 7 || op == 8)
            col += len;
    }
}

char ho_pick_consensus(const uint32_t* k)
{ /* pickConsensusChar (src/consensus/consensus.cpp:18-35) */
    uint32_t best = k[0];
    char ch = 'A';
    if (k[1] > best) best = k[1], ch = 'C';
    if (k[2] > best) best = k[2], ch = 'G';
    if (k[3] > best) best = k[3], ch = 'T';
    if (k[4] > best) best = k[4], ch = 'U';
    return ch;
}

/* ------------------------------------------------------------------ MinHash */

static uint64_t rotl64(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }

static uint32_t bswap32(uint32_t x)
{
    return (x >> 24) | ((x >> 8) & 0xff00u) | ((x << 8) & 0xff0000u) | (x << 24);
}

uint64_t ho_hash2bit(uint64_t code, uint32_t seed32)
{ /* getHash2bit (src/mash/hash.cpp): XXH3 64-bit of the 8 big-endian bytes of
   * code.  XXH3 for a 4..8-byte input: the seed's low word byte-swapped into
   * its high word; the input read as two little-endian words (first word on
   * top); xored with (secret[8..15] ^ secret[16..23]) - seed, where the two
   * secret words are little-endian reads of the default 192-byte secret; then
   * the rrmxmx finaliser with the input length (8). */
    uint64_t seed = seed32;
    seed ^= (uint64_t)bswap32((uint32_t)seed) << 32;
    const uint32_t w_hi = bswap32((uint32_t)(code >> 32)), w_lo = bswap32((uint32_t)code);
    const uint64_t bitflip = 0xc73ab174c5ecd5a2ULL - seed;
    uint64_t h = (((uint64_t)w_hi << 32) + w_lo) ^ bitflip;
    h ^= rotl64(h, 49) ^ rotl64(h, 24);
    h *= 0x9FB21C651E98DF25ULL;
    h ^= (h >> 35) + 8;
    h *= 0x9FB21C651E98DF25ULL;
    return h ^ (h >> 28);
}

static int cmp_u64(const void* a, const void* b)
{
    const uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : x > y;
}

int64_t ho_sketch(const char* seq, int64_t n, int k, int64_t sketch_size, int noncanonical, int seed,
                  uint64_t* out)
{ /* mash::sketchFromSequence (src/mash/mash.cpp:32-117).  Its max-heap plus
   * seen-set keeps exactly the sketch_size smallest distinct hashes seen so
   * far, so the result is the sorted distinct hashes cut to sketch_size. */
    if (k <= 0 || sketch_size <= 0 || n < k || k > 32) return 0;
    /* (1 << 2k) - 1 with the shift count taken mod 64, as x86-64 and AArch64
     * shifts do: at k = 32 the reference's mask is 0 and every code is 0 */
    const uint64_t mask = (1ULL << ((2 * k) & 63)) - 1ULL;
    const int shift = 2 * (k - 1);
    uint64_t* h = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)(n - k + 1));
    int64_t m = 0, valid = 0;
    uint64_t fwd = 0, rev = 0;
    for (int64_t i = 0; i < n; ++i) {
        const unsigned c = nt4((unsigned char)seq[i]); /* mash::nt4_table (include/mash.h:15-32) */
        if (c >= 4) {
            fwd = rev = 0, valid = 0;
            continue;
        }
        fwd = ((fwd << 2) | c) & mask;
        rev = (rev >> 2) | ((uint64_t)(3u ^ c) << shift);
        if (valid < k) ++valid;
        if (valid < k) continue;
        const uint64_t code = noncanonical ? fwd : (fwd < rev ? fwd : rev);
        h[m++] = ho_hash2bit(code, (uint32_t)seed);
    }
    qsort(h, (size_t)m, sizeof(uint64_t), cmp_u64);
    int64_t u = 0;
    for (int64_t i = 0; i < m && u < sketch_size; ++i)
        if (i == 0 || h[i] != h[i - 1]) out[u++] = h[i];
    free(h);
    return u;
}

double ho_jaccard(const uint64_t* a, int64_t na, const uint64_t* b, int64_t nb)
{ /* mash::jaccard (src/mash/mash.cpp:120-164) with the two-pointer
   * intersectionSizeSortedUnique (:204-230) */
    if (na == 0 && nb == 0) return 1.0;
    if (na == 0 || nb == 0) return 0.0;
    int64_t i = 0, j = 0, inter = 0;
    while (i < na && j < nb) {
        if (a[i] < b[j]) ++i;
        else if (b[j] < a[i]) ++j;
        else ++inter, ++i, ++j;
    }
    const int64_t uni = na < nb ? na : nb;
    return (double)inter / (double)uni;
}

int32_t ho_best_reference(const uint64_t* q, int64_t nq, const uint64_t* ref_h, const int64_t* ref_off,
                          int32_t n_refs, double* best_j)
{ /* src/align/ref_aligner.cpp:232-241 */
    double best = -1.0;
    int32_t idx = 0;
    for (int32_t r = 0; r < n_refs; ++r) {
        const double j = ho_jaccard(q, nq, ref_h + ref_off[r], ref_off[r + 1] - ref_off[r]);
        if (j > best) best = j, idx = r;
    }
    if (best_j) *best_j = best;
    return idx;
}
