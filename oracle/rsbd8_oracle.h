/*
 * rsbd8_oracle.h - interface of the oracle (test infrastructure only).
 * A plain-C restatement of the stable LSD radix sort in Radixsortbidi8.hpp;
 * see rsbd8_oracle.c for the reference lines each part follows.
 */
#ifndef RSBD8_ORACLE_H
#define RSBD8_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* key kinds: what std::is_signed_v / std::is_floating_point_v say of the key type */
enum { RSBD8O_KIND_UNSIGNED = 0, RSBD8O_KIND_SIGNED = 1, RSBD8O_KIND_FLOAT = 2 };

typedef struct rsbd8o_desc {
    uint32_t key_bytes;          /* 1, 2, 4 or 8 */
    uint32_t absv, sign, fltp;   /* resolved filter bits (isabsvalue, issignmode, isfltpmode) */
    uint32_t desc, rev;          /* isdescsort and the effective isrevorder */
    uint32_t indirect;           /* 0 keys, 1 pointers to objects, 2 pointers to objects holding a pointer */
    uint32_t pad_;
    int64_t offset1;             /* byte offset of the key (or of the second pointer) in the object */
    int64_t offset2;             /* byte offset of the key behind the second pointer */
} rsbd8o_desc;

/* sortingmode / sortingdirection values -> resolved bits; returns 0 or -1 */
int rsbd8o_resolve(uint32_t kind, uint32_t mode, uint32_t direction, uint32_t indirect,
                   rsbd8o_desc *d);
/* the sort key of raw bits under d (ascending order = output order) */
uint64_t rsbd8o_sortkey(uint64_t bits, uint32_t key_bytes, const rsbd8o_desc *d);
/* stable sort of n elements from in to out (keys, or 8-byte pointers when indirect) */
int rsbd8o_sortcopy(const rsbd8o_desc *d, uint64_t n, const void *in, void *out, unsigned threads);
/* many independent sorts (segments of a batch, requests of a serving run): job i sorts
 * jobs[i].n elements from jobs[i].in to jobs[i].out under *jobs[i].d, each single-threaded,
 * `threads` jobs at a time; returns 0, or the first failing job's code */
typedef struct rsbd8o_job {
    const rsbd8o_desc *d;
    uint64_t n;
    const void *in;
    void *out;
} rsbd8o_job;
int rsbd8o_sortcopy_batch(uint64_t njobs, const rsbd8o_job *jobs, unsigned threads);
/* bit g set when digit g (of digit_bits, 0 = the reference's own width) is skipped */
uint32_t rsbd8o_skipmask(const rsbd8o_desc *d, uint64_t n, const void *in, uint32_t digit_bits);

#ifdef __cplusplus
}
#endif
#endif
