/* oracle_sanitize.c - runs the oracle's C restatement under AddressSanitizer and
 * UndefinedBehaviorSanitizer (built by tests/test_oracle_cpu.py): every key size, every
 * filter combination and direction, direct and through both indirection levels, one and
 * several threads, sizes around the digit-pass and thread-split boundaries.  Each output is
 * checked to be ordered by the oracle's own sort key and to be a permutation of the input. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "rsbd8_oracle.h"

static uint64_t sm(uint64_t *s) {
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static uint64_t get(const unsigned char *p, uint32_t kb) {
    uint64_t v = 0;
    memcpy(&v, p, kb);
    return v;
}

static int cmp_u64(const void *a, const void *b) {
    const uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return x < y ? -1 : x > y;
}

/* sorted by key, and the multiset of raw keys unchanged */
static int check(const rsbd8o_desc *d, uint64_t n, const unsigned char *in, const unsigned char *out) {
    const uint32_t kb = d->key_bytes;
    uint64_t *a = malloc((n + 1) * 8), *b = malloc((n + 1) * 8);
    int ok = 1;
    for (uint64_t i = 0; i < n; ++i) {
        a[i] = get(in + i * kb, kb);
        b[i] = get(out + i * kb, kb);
        if (i && rsbd8o_sortkey(b[i - 1], kb, d) > rsbd8o_sortkey(b[i], kb, d)) ok = 0;
    }
    qsort(a, n, 8, cmp_u64);
    qsort(b, n, 8, cmp_u64);
    if (memcmp(a, b, n * 8)) ok = 0;
    free(a);
    free(b);
    return ok;
}

int main(void) {
    const uint64_t sizes[] = {0, 1, 2, 3, 31, 33, 255, 257, 2049, 65543};
    const uint32_t modes[] = {0, 1, 2, 3, 4, 5, 6, 7, 64, 65, 66};
    uint64_t s = 99;
    int failures = 0;
    for (uint32_t kb = 1; kb <= 8; kb <<= 1)
        for (uint32_t kind = 0; kind < 3; ++kind) {
            if (kind == RSBD8O_KIND_FLOAT && kb < 4) continue;
            for (size_t si = 0; si < sizeof sizes / sizeof *sizes; ++si)
                for (size_t mi = 0; mi < sizeof modes / sizeof *modes; ++mi)
                    for (uint32_t dir = 0; dir < 4; ++dir) {
                        const uint64_t n = sizes[si];
                        rsbd8o_desc d;
                        if (rsbd8o_resolve(kind, modes[mi], dir, 0, &d)) return 2;
                        d.key_bytes = kb;
                        unsigned char *in = malloc(n * kb + 1), *out = malloc(n * kb + 1);
                        for (uint64_t i = 0; i < n * kb; ++i) in[i] = (unsigned char)(sm(&s) & (i % 7 ? 0xFF : 0x03));
                        const unsigned threads = (unsigned)(1 + (si + mi + dir) % 4);
                        if (rsbd8o_sortcopy(&d, n, in, out, threads) || !check(&d, n, in, out)) {
                            fprintf(stderr, "direct failure kb=%u kind=%u n=%llu mode=%u dir=%u\n", kb, kind,
                                    (unsigned long long)n, modes[mi], dir);
                            ++failures;
                        }
                        free(in);
                        free(out);
                    }
        }
    /* indirection: 24-byte objects, key at byte 8; second level through a pointer at byte 16 */
    for (uint32_t level = 1; level <= 2; ++level)
        for (uint32_t dir = 0; dir < 4; ++dir) {
            const uint64_t n = 20011;
            unsigned char *obj = malloc(n * 24);
            uint64_t *keys2 = malloc(n * 8);
            uintptr_t *ptrs = malloc(n * sizeof(uintptr_t)), *outp = malloc(n * sizeof(uintptr_t));
            for (uint64_t i = 0; i < n; ++i) {
                const uint64_t k = sm(&s) % 1000;
                memcpy(obj + i * 24 + 8, &k, 8);
                keys2[i] = k;
                const uint64_t *kp = keys2 + i;
                memcpy(obj + i * 24 + 16, &kp, sizeof kp);
                ptrs[i] = (uintptr_t)(obj + i * 24);
            }
            rsbd8o_desc d;
            if (rsbd8o_resolve(RSBD8O_KIND_UNSIGNED, 64, dir, level, &d)) return 2;
            d.key_bytes = 8;
            d.offset1 = level == 1 ? 8 : 16;
            d.offset2 = 0;
            if (rsbd8o_sortcopy(&d, n, ptrs, outp, 3)) ++failures;
            for (uint64_t i = 1; i < n; ++i) {
                uint64_t a, b;
                memcpy(&a, (const unsigned char *)outp[i - 1] + 8, 8);
                memcpy(&b, (const unsigned char *)outp[i] + 8, 8);
                if ((dir & 1) ? a < b : a > b) {
                    ++failures;
                    break;
                }
            }
            free(obj);
            free(keys2);
            free(ptrs);
            free(outp);
        }
    printf("%s (%d failures)\n", failures ? "FAIL" : "PASS", failures);
    return failures ? 1 : 0;
}
