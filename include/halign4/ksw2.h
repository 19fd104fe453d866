/* ksw2.h - drop-in for HAlign-4's include/ksw2.h on the align-to-center
 * path: the KSW_EZ_* flags, the CIGAR op codes, the ksw_extz_t result record
 * and ksw_extz2_sse, implemented over the GB300 C ABI (hg_ksw_extz2) by
 * libhalign4_dropin.so.  The record layout and the ownership rule (the call
 * (re)allocates ez->cigar with malloc/realloc, growing ez->m_cigar, and the
 * caller frees it) are the reference's.  The other KSW2 entry points the
 * reference header declares (ksw_extz, ksw_extd, ksw_gg, ...) have no
 * implementation in HAlign-4 and are not declared here. */
#ifndef KSW2_H_
#define KSW2_H_

#include <stdint.h>

#define KSW_NEG_INF -0x40000000

#define KSW_EZ_SCORE_ONLY  0x01  /* no alignment path / CIGAR */
#define KSW_EZ_RIGHT       0x02  /* right-align gaps */
#define KSW_EZ_GENERIC_SC  0x04  /* use the full m x m matrix; without it: match/mismatch, last symbol a wildcard */
#define KSW_EZ_APPROX_MAX  0x08  /* approximate maximum */
#define KSW_EZ_APPROX_DROP 0x10  /* approximate z-drop */
#define KSW_EZ_EXTZ_ONLY   0x40  /* extension only */
#define KSW_EZ_REV_CIGAR   0x80  /* CIGAR in reverse order */
#define KSW_EZ_SPLICE_FOR  0x100
#define KSW_EZ_SPLICE_REV  0x200
#define KSW_EZ_SPLICE_FLANK 0x400
#define KSW_EZ_EQX         0x800

#define KSW_CIGAR_MATCH  0
#define KSW_CIGAR_INS    1
#define KSW_CIGAR_DEL    2
#define KSW_CIGAR_N_SKIP 3
#define KSW_CIGAR_EQ     7
#define KSW_CIGAR_X      8

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    uint32_t max:31, zdropped:1;
    int max_q, max_t;   /* coordinates of the maximum */
    int mqe, mqe_t;     /* best score reaching the query end, and its target position */
    int mte, mte_q;     /* best score reaching the target end, and its query position */
    int score;          /* score reaching both ends; may be KSW_NEG_INF */
    int m_cigar, n_cigar;
    int reach_end;
    uint32_t *cigar;
} ksw_extz_t;

/* Affine-gap extension / global alignment of query (qlen codes < m) against
 * target (tlen codes < m) under the m x m matrix mat, gap cost q + l*e, band
 * w (< 0: none), z-drop zdrop (< 0: none) and end bonus; flag = KSW_EZ_*.
 * km is ignored (the reference passes it to its allocator, which is malloc
 * without kalloc).  Runs on the GPU; on a CUDA error the result is left
 * reset (n_cigar 0) and the error text is in hg_last_error(). */
void ksw_extz2_sse(void *km, int qlen, const uint8_t *query, int tlen, const uint8_t *target, int8_t m,
                   const int8_t *mat, int8_t q, int8_t e, int w, int zdrop, int end_bonus, int flag, ksw_extz_t *ez);

#ifdef __cplusplus
}
#endif

/* The reset every call starts from (include/ksw2.h:180-185 in HAlign-4). */
static inline void ksw_reset_extz(ksw_extz_t *ez)
{
    ez->max_q = ez->max_t = ez->mqe_t = ez->mte_q = -1;
    ez->max = 0, ez->score = ez->mqe = ez->mte = KSW_NEG_INF;
    ez->n_cigar = 0, ez->zdropped = 0, ez->reach_end = 0;
}

#endif /* KSW2_H_ */
