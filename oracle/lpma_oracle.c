/*
 * CPU oracle for the LPMA batched edge-update path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker that tests/, the smoke check and the
 * CPU-baseline leg of bench.py use.  The product never links it.
 *
 * It restates, single threaded and slot by slot, the reference algorithm of
 * pkumod/LPMA rpma.cuh (cited per function below): the in-order segment tree
 * laid out one array per level (here the level arrays are concatenated, which
 * is heap order), the reference's locate descent, the level loop with its
 * skip state machine, per-window compaction + merge + even redistribution,
 * eager level-up, resize, rebuild and fill_empty_segs.
 *
 * Extension beyond the reference (whose LPMA has no key delete and keeps
 * duplicate keys): a batch is resolved to a set of updates first
 * (in-batch duplicates collapse, insert of a present key overwrites its
 * value in place as GPMA's handle_del_mod does, gpma.cuh:162-175), and a
 * delete of a present key tombstones its slot (value 0xFF, GPMA's
 * VALUE_NONE) and joins the level loop as a pending update that counts -1
 * toward the window's merge size; executed windows drop tombstones in
 * compaction (gpma.cuh:228 predicate).  For insert-only batches with
 * distinct keys this is exactly the reference.
 *
 * Parity status: the steps that have a host-compilable counterpart in the
 * reference (index macros, density, skip rule, resize height, locate,
 * redistribution) are pinned to that code, compiled from the reference by
 * oracle/ref_host.py; the whole-batch layout is "partially unpinned" (the
 * reference's update loop does not build under CUDA 13) and is pinned by the
 * reference's result checks and a second restatement (tests/golden).
 */
#include "lpma_oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define KEY_NONE (~0ull)
#define VAL_TOMB ((uint8_t)0xFF)
#define TIME_MASK 0x00000000000FFFFFull
#define DST_AND_TIME_MASK 0x000003FFFFFFFFFFull
#define DST_AND_TIME_END 0x000003FFFFEFFFFFull
#define SRC_SHIFT 42
#define DST_SHIFT 20
#define DST_MASK 0x000003FFFFF00000ull
#define NBR_END 0x003FFFFEu
#define MAX_HEIGHT 24

enum { K_INS = 0, K_DEL = 1 };

struct OPma {
    uint32_t H;
    uint32_t V;
    int skip_rule;
    uint64_t *keys; /* heap order: level i starts at slot 32*(2^i - 1) */
    uint8_t *vals;
    uint32_t *sent; /* physical slot of vertex v's sentinel */
    uint32_t lower[32], upper[32];
};

typedef struct {
    uint64_t key;
    uint64_t node; /* linear slot index of the window start */
    uint8_t val;
    uint8_t kind;
    uint8_t applied;
} Upd;

typedef struct {
    Upd *u;
    size_t n;
} Pending;

/* ------------------------------------------------------------------ */
/* index algebra, rpma.cuh:98-134                                       */
/* ------------------------------------------------------------------ */
static uint32_t ref_lls(uint32_t x) {
    uint32_t r = 1;
    if (!(x & 0x0000ffffu)) x >>= 16, r += 16;
    if (!(x & 0x000000ffu)) x >>= 8, r += 8;
    if (!(x & 0x0000000fu)) x >>= 4, r += 4;
    if (!(x & 0x00000003u)) x >>= 2, r += 2;
    if (!(x & 0x00000001u)) x >>= 1, r += 1;
    return r;
}
uint32_t opma_get_idx(uint32_t L, uint32_t H) { return H + 1 - ref_lls((L >> 5) + 1); }
uint32_t opma_get_lane(uint32_t L, uint32_t I, uint32_t H) {
    return (((((L >> 5) + 1) >> (H - I)) - 1) >> 1 << 5) + (L % 32);
}
uint32_t opma_get_linear_idx(uint32_t I, uint32_t lane, uint32_t H) {
    return (32u << (H - I)) - 32 + ((lane >> 5) << (H - I + 1) << 5);
}

static inline uint64_t nseg_of(uint32_t H) { return (2ull << H) - 1; }
static inline uint64_t nslots_of(uint32_t H) { return 32ull * nseg_of(H); }
static inline uint64_t lvl_base(uint32_t i) { return 32ull * ((1ull << i) - 1); }

/* linear slot -> physical (heap) slot; 64-bit form of GET_IDX/GET_LANE */
static inline uint64_t phys_of(uint64_t L, uint32_t H) {
    uint64_t s1 = (L >> 5) + 1;
    uint32_t t = (uint32_t)__builtin_ctzll(s1);
    uint32_t i = H - t;
    uint64_t pos = s1 >> (t + 1);
    return lvl_base(i) + 32 * pos + (L & 31);
}

/* recalculate_density, rpma.cuh:137-168: lower = trunc(0.42 * 32 * 2^i) */
void opma_density_table(uint32_t *lower, uint32_t *upper, int n) {
    uint64_t len = 32;
    for (int i = 0; i < n; i++) {
        double d = 0.42 * (double)len;
        lower[i] = (uint32_t)d;
        upper[i] = (uint32_t)len;
        len <<= 1;
    }
}

/* skip state machine, rpma.cuh:1609-1619 */
void opma_skip_table(uint32_t H, uint8_t *out, int n) {
    int skip = 0;
    for (int level = 0; level < n; level++) {
        uint32_t lv = (uint32_t)level;
        if (lv == 4 || lv == H / 3) skip = 1;
        if (lv == (uint32_t)(H / 3 - 1u) || lv == H + 1) skip = 0;
        out[level] = (uint8_t)skip;
    }
}

void opma_redistribute_counts(uint64_t f, uint64_t m, uint32_t *counts) {
    for (uint64_t k = 0; k < f; k++) counts[k] = 0;
    for (uint64_t i = 0; i < m; i++) counts[(f * i) / m]++;
}

/* ------------------------------------------------------------------ */
/* small utilities                                                      */
/* ------------------------------------------------------------------ */
uint64_t opma_mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* LSD radix sort of u64 keys with an optional u64 payload, 8-bit digits,
 * constant bytes skipped.  Stable. */
static void radix_sort_u64(uint64_t *k, uint64_t *v, uint64_t n) {
    if (n < 2) return;
    uint64_t *tk = (uint64_t *)malloc(n * sizeof(uint64_t));
    uint64_t *tv = v ? (uint64_t *)malloc(n * sizeof(uint64_t)) : NULL;
    uint64_t and_all = ~0ull, or_all = 0;
    for (uint64_t i = 0; i < n; i++) and_all &= k[i], or_all |= k[i];
    uint64_t diff = and_all ^ or_all;
    uint64_t *sk = k, *sv = v, *dk = tk, *dv = tv;
    for (int pass = 0; pass < 8; pass++) {
        int sh = pass * 8;
        if (!((diff >> sh) & 0xFF)) continue;
        uint64_t cnt[257];
        memset(cnt, 0, sizeof(cnt));
        for (uint64_t i = 0; i < n; i++) cnt[((sk[i] >> sh) & 0xFF) + 1]++;
        for (int d = 0; d < 256; d++) cnt[d + 1] += cnt[d];
        for (uint64_t i = 0; i < n; i++) {
            uint64_t o = cnt[(sk[i] >> sh) & 0xFF]++;
            dk[o] = sk[i];
            if (v) dv[o] = sv[i];
        }
        uint64_t *t = sk; sk = dk; dk = t;
        t = sv; sv = dv; dv = t;
    }
    if (sk != k) {
        memcpy(k, sk, n * sizeof(uint64_t));
        if (v) memcpy(v, sv, n * sizeof(uint64_t));
    }
    free(tk);
    free(tv);
}

/* ------------------------------------------------------------------ */
/* structure maintenance                                                */
/* ------------------------------------------------------------------ */
static int set_height(OPma *p, uint32_t h, int clear_all) {
    uint64_t old_n = nslots_of(p->H), new_n = nslots_of(h);
    uint64_t *k = (uint64_t *)realloc(p->keys, new_n * sizeof(uint64_t));
    uint8_t *v = (uint8_t *)realloc(p->vals, new_n);
    if (!k || !v) return -1;
    p->keys = k;
    p->vals = v;
    if (clear_all) {
        memset(p->keys, 0xFF, new_n * sizeof(uint64_t));
        memset(p->vals, 0, new_n);
    } else if (new_n > old_n) {
        /* alloc_or_del_levels, rpma.cuh:1396-1415: new levels empty */
        memset(p->keys + old_n, 0xFF, (new_n - old_n) * sizeof(uint64_t));
        memset(p->vals + old_n, 0, new_n - old_n);
    }
    p->H = h;
    return 0;
}

static inline int is_sentinel(uint64_t key) { return (key & DST_AND_TIME_MASK) == DST_AND_TIME_END; }

static inline int kept(uint64_t key, uint8_t val, uint32_t thres) {
    return key != KEY_NONE && (key & TIME_MASK) >= (uint64_t)thres && val != VAL_TOMB;
}

/* even redistribution, rpma.cuh:676-695 / 964-983 */
static void redistribute(OPma *p, const uint64_t *mk, const uint8_t *mv, uint64_t m, uint64_t w,
                         uint64_t width) {
    uint64_t f = width / 32;
    for (uint64_t L = w; L < w + width; L++) p->keys[phys_of(L, p->H)] = KEY_NONE;
    for (uint64_t i = 0; i < m; i++) {
        uint64_t seg = (f * i) / m;
        uint64_t lane = ((f * i) % m) / f;
        uint64_t ph = phys_of(w + seg * 32 + lane, p->H);
        p->keys[ph] = mk[i];
        p->vals[ph] = mv[i];
        if (is_sentinel(mk[i])) {
            uint32_t row = (uint32_t)(mk[i] >> SRC_SHIFT);
            if (row < p->V) p->sent[row] = (uint32_t)ph;
        }
    }
}

static uint64_t count_live(const OPma *p, uint32_t thres) {
    uint64_t n = nslots_of(p->H), c = 0;
    for (uint64_t i = 0; i < n; i++) c += kept(p->keys[i], p->vals[i], thres);
    return c;
}

/* resize_rpma, rpma.cuh:1301-1354: least h with 32*(2^(h+1)-1) >= count */
static uint32_t min_height(uint64_t cnt) {
    uint32_t h = 0;
    while (nslots_of(h) < cnt) h++;
    return h;
}

/* compaction of a linear slot range into (k, v), kept predicate */
static uint64_t compact_range(const OPma *p, uint64_t w, uint64_t width, uint32_t thres, uint64_t *k,
                              uint8_t *v) {
    uint64_t c = 0;
    for (uint64_t L = w; L < w + width; L++) {
        uint64_t ph = phys_of(L, p->H);
        if (kept(p->keys[ph], p->vals[ph], thres)) {
            k[c] = p->keys[ph];
            v[c] = p->vals[ph];
            c++;
        }
    }
    return c;
}

/* locate_leaf_kernel, rpma.cuh:254-316: descend the in-order segment tree;
 * returns GET_LINEAR_IDX of the stop segment (a linear slot index) */
static uint64_t locate(const OPma *p, uint64_t key) {
    uint32_t H = p->H, idx = 0;
    uint64_t lane = 0;
    while (idx < H) {
        const uint64_t *lv = p->keys + lvl_base(idx);
        if (lv[lane] == KEY_NONE) break;
        if (lv[lane] > key) {
            ++idx;
            lane <<= 1;
            continue;
        }
        uint32_t l = 0, r = 31;
        while (l < r) {
            uint32_t mid = (l + r + 1) >> 1;
            if (lv[lane + mid] == KEY_NONE)
                r = mid - 1;
            else
                l = mid;
        }
        if (key > lv[lane + l]) {
            ++idx;
            lane = (lane << 1) + 32;
        } else
            break;
    }
    return (32ull << (H - idx)) - 32 + ((lane >> 5) << (H - idx + 1) << 5);
}

/* ------------------------------------------------------------------ */
/* level loop, rpma.cuh:1611-1657 (first loop) and 1686-1703 (second)   */
/* ------------------------------------------------------------------ */
static void run_level_loop(OPma *p, Pending *P, uint32_t thres, int use_skip, int eager, OPmaStats *st,
                           uint64_t *bk, uint8_t *bv, uint64_t *mk, uint8_t *mv) {
    int skip = 0;
    for (uint32_t level = 0; level <= p->H + 1 && P->n > 0; ++level) {
        uint32_t H = p->H;
        if (use_skip) {
            if (level == 4 || level == H / 3) skip = 1;
            if (level == (uint32_t)(H / 3 - 1u) || level == H + 1) skip = 0;
        }
        uint64_t width = 32ull << level;
        uint32_t lower = p->lower[level];
        uint64_t total = 32ull << (H + 1);
        size_t i = 0;
        while (i < P->n) {
            uint64_t node = P->u[i].node;
            size_t j = i;
            while (j < P->n && P->u[j].node == node) j++;
            uint64_t ww = width, up = p->upper[level];
            int ok = 1;
            /* clip the last window, rpma.cuh:787-792 / 1150-1155 */
            if (node + ww >= total) {
                ww -= 32;
                up -= 32;
                if (ww == 0) ok = 0;
            }
            /* big grain honours skip, rpma.cuh:1167 */
            if (ok && ww > 1024 && skip) ok = 0;
            if (ok) {
                uint64_t a = compact_range(p, node, ww, thres, bk, bv);
                uint64_t nins = 0;
                for (size_t t = i; t < j; t++) nins += (P->u[t].kind == K_INS);
                uint64_t m = a + nins;
                if (lower <= m && m <= up) {
                    /* mergesmallk / pathBig_k: stable merge, ties take A */
                    uint64_t x = 0, y = 0, o = 0;
                    size_t t = i;
                    while (x < a || t < j) {
                        while (t < j && P->u[t].kind != K_INS) t++;
                        if (t < j && (x >= a || P->u[t].key < bk[x])) {
                            mk[o] = P->u[t].key;
                            mv[o] = P->u[t].val;
                            t++;
                        } else if (x < a) {
                            mk[o] = bk[x];
                            mv[o] = bv[x];
                            x++;
                        } else
                            break;
                        o++;
                    }
                    (void)y;
                    redistribute(p, mk, mv, m, node, ww);
                    for (size_t q = i; q < j; q++) P->u[q].applied = 1;
                    if (st && level < 32) {
                        st->win_count[level]++;
                        st->win_slots[level] += ww;
                    }
                    if (level == H + 1 && st) st->root_executed = 1;
                }
            }
            i = j;
        }
        /* compact_insertions + up_level_kernel, rpma.cuh:1632-1642 */
        size_t o = 0;
        for (size_t q = 0; q < P->n; q++)
            if (!P->u[q].applied) {
                P->u[o] = P->u[q];
                P->u[o].node &= ~(32ull << level);
                o++;
            }
        P->n = o;
        /* eager level-up when the root absorbed everything, rpma.cuh:1646-1653 */
        if (eager && level == H + 1 && P->n == 0) {
            if (st) st->levelup = 1;
            uint64_t c = count_live(p, thres);
            uint32_t h = min_height(c) + 1;
            if (h > p->H) {
                set_height(p, h, 0);
                if (st) st->eager_levelup = 1;
            }
        }
    }
}


/* rebuild_rpma, rpma.cuh:1417-1472: compact all, add pending inserts, sort,
 * redistribute over the whole array at height h */
static int rebuild(OPma *p, uint32_t h, Pending *P, uint32_t thres) {
    uint64_t n = nslots_of(p->H);
    uint64_t cap = n + P->n;
    uint64_t *k = (uint64_t *)malloc(cap * sizeof(uint64_t));
    uint8_t *v = (uint8_t *)malloc(cap);
    uint64_t *mk = (uint64_t *)malloc(cap * sizeof(uint64_t));
    uint8_t *mv = (uint8_t *)malloc(cap);
    if (!k || !v || !mk || !mv) return -1;
    uint64_t a = compact_range(p, 0, n, thres, k, v);
    /* pending inserts are sorted by key; the stored sequence is sorted; merge */
    uint64_t x = 0, o = 0;
    size_t t = 0;
    while (x < a || t < P->n) {
        while (t < P->n && P->u[t].kind != K_INS) t++;
        if (t < P->n && (x >= a || P->u[t].key < k[x])) {
            mk[o] = P->u[t].key;
            mv[o] = P->u[t].val;
            t++;
        } else if (x < a) {
            mk[o] = k[x];
            mv[o] = v[x];
            x++;
        } else
            break;
        o++;
    }
    if (set_height(p, h, 1)) return -1;
    redistribute(p, mk, mv, o, 0, nslots_of(h));
    P->n = 0;
    free(k);
    free(v);
    free(mk);
    free(mv);
    return 0;
}

/* fill_empty_segs, rpma.cuh:1474-1530 */
static int fill_empty_segs(OPma *p, uint32_t thres, OPmaStats *st) {
    uint32_t H = p->H;
    uint64_t base = (1ull << (H - 1)) - 1, cnt = 1ull << (H - 1);
    int empty = 0;
    for (uint64_t j = base; j < base + cnt && !empty; j++) {
        int any = 0;
        for (int l = 0; l < 32; l++) any |= (p->keys[32 * j + l] != KEY_NONE);
        if (!any) empty = 1;
    }
    if (!empty) return 0;
    uint64_t n = nslots_of(H);
    uint64_t *k = (uint64_t *)malloc(n * sizeof(uint64_t));
    uint8_t *v = (uint8_t *)malloc(n);
    if (!k || !v) return -1;
    uint64_t a = compact_range(p, 0, n, thres, k, v);
    redistribute(p, k, v, a, 0, n);
    free(k);
    free(v);
    if (st) st->fill_empty = 1;
    return 0;
}

/* ------------------------------------------------------------------ */
/* public API                                                           */
/* ------------------------------------------------------------------ */
typedef struct {
    uint64_t key;
    uint32_t order;
    uint8_t kind;
    uint8_t val;
} Ent;

static int cmp_ent(const void *a, const void *b) {
    const Ent *x = (const Ent *)a, *y = (const Ent *)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    if (x->kind != y->kind) return x->kind < y->kind ? -1 : 1;
    return x->order < y->order ? -1 : (x->order > y->order);
}

static int update_impl(OPma *p, const uint64_t *ins, const uint8_t *ins_vals, size_t n_ins, const uint64_t *del,
                       size_t n_del, uint32_t thres, OPmaStats *st, int internal) {
    OPmaStats dummy;
    if (!st) st = &dummy;
    memset(st, 0, sizeof(*st));
    st->height_before = p->H;
    size_t n = n_ins + n_del;
    if (n == 0) {
        st->height_after = p->H;
        return 0;
    }
    /* validation (the product rejects the same inputs) */
    for (size_t i = 0; i < n_ins; i++) {
        if (ins[i] == KEY_NONE || (ins[i] >> SRC_SHIFT) >= p->V) return -2;
        if (!(internal && is_sentinel(ins[i])) && ((ins[i] & DST_MASK) >> DST_SHIFT) >= p->V) return -2;
        if (ins_vals && ins_vals[i] == VAL_TOMB) return -2;
        if ((ins[i] & TIME_MASK) < (uint64_t)thres) return -2; /* expired on arrival */
    }
    for (size_t i = 0; i < n_del; i++) {
        if (del[i] == KEY_NONE || (del[i] >> SRC_SHIFT) >= p->V || is_sentinel(del[i])) return -2;
        if (((del[i] & DST_MASK) >> DST_SHIFT) >= p->V) return -2;
    }
    /* resolve the batch into a set of updates: sorted by key, inserts of a
     * key before its deletes; an insert wins over a delete of the same key
     * and the last insert of a key gives its value */
    Ent *e = (Ent *)malloc(n * sizeof(Ent));
    Upd *u = (Upd *)malloc(n * sizeof(Upd));
    if (!e || !u) return -1;
    for (size_t i = 0; i < n_ins; i++) {
        e[i].key = ins[i];
        e[i].order = (uint32_t)i;
        e[i].kind = K_INS;
        e[i].val = ins_vals ? ins_vals[i] : 1;
    }
    for (size_t i = 0; i < n_del; i++) {
        e[n_ins + i].key = del[i];
        e[n_ins + i].order = (uint32_t)i;
        e[n_ins + i].kind = K_DEL;
        e[n_ins + i].val = 0;
    }
    qsort(e, n, sizeof(Ent), cmp_ent);
    Pending P = {u, 0};
    for (size_t i = 0; i < n;) {
        size_t j = i;
        while (j < n && e[j].key == e[i].key) j++;
        const Ent *rep = &e[i];
        if (e[i].kind == K_INS) {
            size_t q = i;
            while (q + 1 < j && e[q + 1].kind == K_INS) q++;
            rep = &e[q];
        }
        st->n_noop += (uint32_t)(j - i - 1);
        /* locate + membership scan of the stop segment (handle_del_mod) */
        uint64_t node = locate(p, rep->key);
        uint64_t ph0 = phys_of(node, p->H);
        int64_t hit = -1;
        for (int l = 0; l < 32; l++)
            if (p->keys[ph0 + l] == rep->key) {
                hit = (int64_t)(ph0 + l);
                break;
            }
        if (rep->kind == K_INS) {
            if (hit >= 0) {
                p->vals[hit] = rep->val;
                st->n_upserts++;
            } else {
                P.u[P.n].key = rep->key;
                P.u[P.n].val = rep->val;
                P.u[P.n].kind = K_INS;
                P.u[P.n].node = node;
                P.u[P.n].applied = 0;
                P.n++;
                st->n_ins_applied++;
            }
        } else {
            if (hit >= 0 && (rep->key & TIME_MASK) >= thres && p->vals[hit] != VAL_TOMB) {
                p->vals[hit] = VAL_TOMB;
                P.u[P.n].key = rep->key;
                P.u[P.n].val = 0;
                P.u[P.n].kind = K_DEL;
                P.u[P.n].node = node;
                P.u[P.n].applied = 0;
                P.n++;
                st->n_del_applied++;
            } else
                st->n_noop++;
        }
        i = j;
    }
    free(e);

    uint64_t nsl = nslots_of(p->H) + 64;
    uint64_t scratch = nsl + P.n + 64;
    uint64_t *bk = (uint64_t *)malloc(scratch * sizeof(uint64_t) * 2);
    uint8_t *bv = (uint8_t *)malloc(scratch * 2);
    if (!bk || !bv) return -1;
    uint64_t *mk = bk + scratch;
    uint8_t *mv = bv + scratch;
    int rc = 0;
    if (P.n > 0) run_level_loop(p, &P, thres, p->skip_rule, 1, st, bk, bv, mk, mv);
    if (P.n > 0) {
        /* overflow, rpma.cuh:1662-1712 */
        st->overflow = 1;
        st->levelup = 1;
        uint64_t c = count_live(p, thres);
        for (size_t q = 0; q < P.n; q++) c += (P.u[q].kind == K_INS);
        uint32_t h = min_height(c);
        if (h > MAX_HEIGHT) {
            rc = -3;
        } else if (h == p->H + 1) {
            st->levelup_path = 1;
            set_height(p, h, 0);
            free(bk);
            free(bv);
            nsl = nslots_of(p->H) + 64;
            scratch = nsl + P.n + 64;
            bk = (uint64_t *)malloc(scratch * sizeof(uint64_t) * 2);
            bv = (uint8_t *)malloc(scratch * 2);
            mk = bk + scratch;
            mv = bv + scratch;
            for (size_t q = 0; q < P.n; q++) P.u[q].node = locate(p, P.u[q].key);
            run_level_loop(p, &P, thres, 0, 0, st, bk, bv, mk, mv);
            if (P.n > 0) {
                /* the reference asserts here (rpma.cuh:1704); rebuild instead */
                uint64_t c2 = count_live(p, thres);
                for (size_t q = 0; q < P.n; q++) c2 += (P.u[q].kind == K_INS);
                st->rebuilt = 1;
                rc = rebuild(p, min_height(c2), &P, thres);
            } else if (p->H > 0) {
                rc = fill_empty_segs(p, thres, st);
            }
        } else {
            /* h < H or h > H+1 rebuild; h == H (the reference asserts,
             * rpma.cuh:1710) also rebuilds at h */
            st->rebuilt = 1;
            rc = rebuild(p, h, &P, thres);
        }
    }
    free(bk);
    free(bv);
    free(u);
    st->height_after = p->H;
    return rc;
}

int opma_update(OPma *p, const uint64_t *ins, const uint8_t *ins_vals, size_t n_ins, const uint64_t *del,
                size_t n_del, uint32_t thres, OPmaStats *st) {
    return update_impl(p, ins, ins_vals, n_ins, del, n_del, thres, st, 0);
}

OPma *opma_create(uint32_t V, int skip_rule) {
    if (V == 0 || V > NBR_END) return NULL;
    OPma *p = (OPma *)calloc(1, sizeof(OPma));
    if (!p) return NULL;
    p->V = V;
    p->skip_rule = skip_rule;
    p->H = 0;
    p->keys = (uint64_t *)malloc(32 * sizeof(uint64_t));
    p->vals = (uint8_t *)calloc(32, 1);
    p->sent = (uint32_t *)calloc(V, sizeof(uint32_t));
    memset(p->keys, 0xFF, 32 * sizeof(uint64_t));
    opma_density_table(p->lower, p->upper, 32);
    uint64_t *s = (uint64_t *)malloc((size_t)V * sizeof(uint64_t));
    uint8_t *sv = (uint8_t *)calloc(V, 1);
    for (uint32_t v = 0; v < V; v++) s[v] = ((uint64_t)v << SRC_SHIFT) + DST_AND_TIME_END;
    int rc = update_impl(p, s, sv, V, NULL, 0, 0, NULL, 1);
    free(s);
    free(sv);
    if (rc) {
        opma_destroy(p);
        return NULL;
    }
    return p;
}

void opma_destroy(OPma *p) {
    if (!p) return;
    free(p->keys);
    free(p->vals);
    free(p->sent);
    free(p);
}

uint32_t opma_height(const OPma *p) { return p->H; }
uint64_t opma_num_slots(const OPma *p) { return nslots_of(p->H); }
uint64_t opma_num_items(const OPma *p) {
    uint64_t n = nslots_of(p->H), c = 0;
    for (uint64_t i = 0; i < n; i++) c += (p->keys[i] != KEY_NONE);
    return c;
}

int opma_layout(const OPma *p, uint64_t *keys, uint8_t *vals, size_t cap) {
    uint64_t n = nslots_of(p->H);
    if (cap < n) return -1;
    memcpy(keys, p->keys, n * sizeof(uint64_t));
    for (uint64_t i = 0; i < n; i++) vals[i] = p->keys[i] == KEY_NONE ? 0 : p->vals[i];
    return 0;
}

int opma_sentinel_slots(const OPma *p, uint32_t *out, size_t cap) {
    if (cap < p->V) return -1;
    memcpy(out, p->sent, (size_t)p->V * sizeof(uint32_t));
    return 0;
}

int64_t opma_export_sorted(const OPma *p, uint64_t *keys, uint8_t *vals, size_t cap) {
    uint64_t nseg = nseg_of(p->H), c = 0;
    for (uint64_t s = 0; s < nseg; s++) {
        uint64_t ph = phys_of(s * 32, p->H);
        for (int l = 0; l < 32; l++) {
            uint64_t k = p->keys[ph + l];
            if (k == KEY_NONE) continue;
            if (c < cap) {
                keys[c] = k;
                if (vals) vals[c] = p->vals[ph + l];
            }
            c++;
        }
    }
    return (int64_t)c;
}

int64_t opma_csr(const OPma *p, uint32_t *row_offset, uint32_t *col_index, uint8_t *values, size_t cap) {
    uint64_t nseg = nseg_of(p->H), c = 0;
    row_offset[0] = 0;
    for (uint64_t s = 0; s < nseg; s++) {
        uint64_t ph = phys_of(s * 32, p->H);
        for (int l = 0; l < 32; l++) {
            uint64_t k = p->keys[ph + l];
            if (k == KEY_NONE) continue;
            uint32_t src = (uint32_t)(k >> SRC_SHIFT);
            uint32_t dst = (uint32_t)((k & DST_MASK) >> DST_SHIFT);
            if (c < cap) {
                if (dst == NBR_END) {
                    col_index[c] = src;
                    if (values) values[c] = VAL_TOMB;
                    row_offset[src + 1] = (uint32_t)(c + 1);
                } else {
                    col_index[c] = dst;
                    if (values) values[c] = p->vals[ph + l];
                }
            }
            c++;
        }
    }
    row_offset[p->V] = (uint32_t)c;
    return (int64_t)c;
}

/* ------------------------------------------------------------------ */
/* generators                                                           */
/* ------------------------------------------------------------------ */
void opma_rmat_raw(uint64_t seed, uint32_t scale, uint64_t n_edges, uint32_t ta, uint32_t tab, uint32_t tabc,
                   uint64_t *out) {
    uint64_t s0 = opma_mix64(seed);
    for (uint64_t e = 0; e < n_edges; e++) {
        uint64_t src = 0, dst = 0;
        for (uint32_t b = 0; b < scale; b++) {
            uint32_t r = (uint32_t)(opma_mix64(s0 ^ ((e << 6) | b)) >> 32);
            uint64_t sb = r >= tab, db = (r >= ta && r < tab) || r >= tabc;
            src = (src << 1) | sb;
            dst = (dst << 1) | db;
        }
        out[e] = (src << SRC_SHIFT) | (dst << DST_SHIFT);
    }
}

uint64_t opma_dedup(uint64_t *keys, uint64_t n) {
    uint64_t o = 0;
    for (uint64_t i = 0; i < n; i++) {
        uint64_t src = keys[i] >> SRC_SHIFT, dst = (keys[i] & DST_MASK) >> DST_SHIFT;
        if (src != dst) keys[o++] = keys[i];
    }
    radix_sort_u64(keys, NULL, o);
    uint64_t w = 0;
    for (uint64_t i = 0; i < o; i++)
        if (w == 0 || keys[w - 1] != keys[i]) keys[w++] = keys[i];
    return w;
}

void opma_shuffle(uint64_t seed, uint64_t *keys, uint64_t n) {
    /* (hash, key) order: sort by key first, then stable by hash */
    uint64_t *h = (uint64_t *)malloc(n * sizeof(uint64_t));
    radix_sort_u64(keys, NULL, n);
    for (uint64_t i = 0; i < n; i++) h[i] = opma_mix64(seed ^ keys[i]);
    radix_sort_u64(h, keys, n);
    free(h);
}

/* ------------------------------------------------------------------ */
/* test hooks: single steps of the oracle, for the comparison with the   */
/* reference's own functions compiled for the host (oracle/ref_host.py)  */
/* ------------------------------------------------------------------ */
int opma_locate_keys(const OPma *p, const uint64_t *keys, size_t n, uint32_t *out) {
    for (size_t i = 0; i < n; i++) out[i] = (uint32_t)locate(p, keys[i]);
    return 0;
}

int opma_redistribute_window(uint32_t H, uint32_t V, uint64_t node, uint64_t width, const uint64_t *mk,
                             const uint8_t *mv, uint64_t m, uint64_t *keys, uint8_t *vals, uint32_t *sent) {
    OPma t;
    memset(&t, 0, sizeof(t));
    t.H = H;
    t.V = V;
    t.keys = keys;
    t.vals = vals;
    t.sent = sent;
    if (m > width || node + width > nslots_of(H) + 32) return -1;
    redistribute(&t, mk, mv, m, node, width);
    return 0;
}

/* resize_rpma's height for `count` items, plus one when the root absorbed */
uint32_t opma_resize_height(uint64_t count, int reach_root) { return min_height(count) + (reach_root ? 1u : 0u); }

/* ================================================================== */
/* GPMA (gpma.cuh): one flat packed memory array                        */
/* ================================================================== */
/* Keys src << 32 | dst; the sentinel of row v is v << 32 | 0xFFFFFFFF
 * (col_idx_none, gpma.cuh:826-834); two KEY_MAX guards (init_gpma,
 * gpma.cuh:818-823) stay at the end.  size = segment_length << tree_height,
 * a power of two.  A delete is an update with value VALUE_NONE: it
 * tombstones a present key in place and never enters the level loop
 * (handle_del_mod, gpma.cuh:162-175). */
#define G_KEY_MAX 0xFFFFFFFFFFFFFFFEull
#define G_COL_NONE 0xFFFFFFFFull
#define G_SIGNIFICANT 5000000u

struct OGpma {
    uint32_t V;
    uint64_t size;
    uint32_t seg, h;
    uint64_t *keys;
    uint8_t *vals;
    uint32_t *row; /* row_offset: row_offset[v + 1] = slot of v's sentinel */
    double dlow;   /* density_lower_thres_root (gpma.cuh:52) */
    uint32_t lower[40], upper[40];
};

static uint32_t g_fls(uint32_t x) { return x ? 32u - (uint32_t)__builtin_clz(x) : 0u; }

/* recalculate_density, gpma.cuh:102-131 */
static void g_density(OGpma *g) {
    uint32_t len = g->seg;
    for (uint32_t i = 0; i <= g->h && i < 40; i++) {
        g->lower[i] = (uint32_t)(g->dlow * (double)len);
        g->upper[i] = len;
        len <<= 1;
    }
}

/* the size rule of resize_gpma, gpma.cuh:706-711 */
static void g_size_rule(uint64_t merge, uint64_t *size, uint32_t *seg, uint32_t *h) {
    uint64_t t = 4;
    while ((double)t < (double)merge) t <<= 1;
    *size = t;
    *seg = 1u << (g_fls(g_fls((uint32_t)t)) - 1);
    *h = g_fls((uint32_t)(t / *seg)) - 1;
}

static inline int g_kept(uint64_t k, uint8_t v) { return k != KEY_NONE && v != VAL_TOMB; }
static inline int g_is_sentinel(uint64_t k) { return (k & G_COL_NONE) == G_COL_NONE && k != KEY_NONE; }

/* redispatch_kernel, gpma.cuh:428-452: item i of m to segment f*i/m, lane
 * (f*i % m)/f of the window [node, node + width); the callers leave every
 * other key of the window empty (block_compact_kernel + the first-m clear
 * of block_redispatch_kernel, or memset_kernel) */
static void g_spread(OGpma *g, const uint64_t *k, const uint8_t *v, uint64_t m, uint64_t node, uint64_t width) {
    const uint64_t frac = width / g->seg;
    for (uint64_t i = 0; i < width; i++) g->keys[node + i] = KEY_NONE;
    for (uint64_t i = 0; i < m; i++) {
        const uint64_t si = frac * i / m, lane = frac * i % m / frac;
        const uint64_t p = node + si * g->seg + lane;
        g->keys[p] = k[i];
        g->vals[p] = v[i];
        if (g_is_sentinel(k[i])) {
            const uint64_t row = k[i] >> 32;
            if (row < g->V) g->row[row + 1] = (uint32_t)p;
        }
    }
}

/* locate_leaf_kernel, gpma.cuh:177-200: binary search over the first slot
 * of the segments */
static uint64_t g_locate(const OGpma *g, uint64_t key) {
    uint64_t prefix = 0, bit = ((uint64_t)g->seg << g->h) >> 1;
    while (g->seg <= bit) {
        if (g->keys[prefix | bit] <= key) prefix |= bit;
        bit >>= 1;
    }
    return prefix;
}

typedef struct {
    uint64_t key;
    uint64_t idx;
    uint8_t val;
} GItem;

static int cmp_gitem(const void *a, const void *b) {
    const GItem *x = (const GItem *)a, *y = (const GItem *)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return x->idx < y->idx ? -1 : (x->idx > y->idx);
}

/* the window's kept items followed by its inserts, sorted stably by key
 * (the block radix sort of block_redispatch_kernel / cub_sort_key_value) */
static uint64_t g_merge_sorted(GItem *buf, uint64_t n, uint64_t *k, uint8_t *v) {
    qsort(buf, n, sizeof(GItem), cmp_gitem);
    for (uint64_t i = 0; i < n; i++) k[i] = buf[i].key, v[i] = buf[i].val;
    return n;
}

/* resize_gpma, gpma.cuh:694-718: compact the whole array in order, choose
 * the size for compacted + pending, reallocate (copying) */
static int g_resize(OGpma *g, uint64_t pending) {
    uint64_t c = 0;
    for (uint64_t i = 0; i < g->size; i++)
        if (g_kept(g->keys[i], g->vals[i])) {
            g->keys[c] = g->keys[i];
            g->vals[c] = g->vals[i];
            c++;
        }
    uint64_t ns;
    uint32_t seg, h;
    g_size_rule(c + pending, &ns, &seg, &h);
    uint64_t *k = (uint64_t *)malloc(ns * sizeof(uint64_t));
    uint8_t *v = (uint8_t *)calloc(ns, 1);
    if (!k || !v) return -1;
    for (uint64_t i = 0; i < ns; i++) k[i] = i < c ? g->keys[i] : KEY_NONE;
    for (uint64_t i = 0; i < c && i < ns; i++) v[i] = g->vals[i];
    free(g->keys);
    free(g->vals);
    g->keys = k;
    g->vals = v;
    g->size = ns;
    g->seg = seg;
    g->h = h;
    g_density(g);
    return 0;
}

/* every kept item plus the pending inserts, sorted and spread over the whole
 * array: the root rebalance after resize_gpma (gpma.cuh:801-813) and
 * significant_insert (gpma.cuh:720-744; its scratch is value-initialised,
 * so there every empty slot holds key 0 -- here empty slots hold KEY_NONE,
 * as after every other rebalance) */
static int g_spread_all(OGpma *g, const Upd *u, size_t n) {
    if (g_resize(g, n)) return -1;
    uint64_t c = 0;
    while (c < g->size && g->keys[c] != KEY_NONE) c++;
    GItem *buf = (GItem *)malloc((c + n + 1) * sizeof(GItem));
    uint64_t *mk = (uint64_t *)malloc((c + n + 1) * sizeof(uint64_t));
    uint8_t *mv = (uint8_t *)malloc(c + n + 1);
    if (!buf || !mk || !mv) return -1;
    for (uint64_t i = 0; i < c; i++) buf[i] = (GItem){g->keys[i], i, g->vals[i]};
    for (size_t q = 0; q < n; q++) buf[c + q] = (GItem){u[q].key, c + q, u[q].val};
    uint64_t m = g_merge_sorted(buf, c + n, mk, mv);
    if (m < g->lower[g->h] || m > g->upper[g->h]) return -4; /* the root check after a resize always passes */
    g_spread(g, mk, mv, m, 0, g->size);
    free(buf);
    free(mk);
    free(mv);
    return 0;
}

static int g_build_from(OGpma *g, const uint64_t *k, const uint8_t *v, uint64_t n) {
    Upd *u = (Upd *)calloc(n + 1, sizeof(Upd));
    if (!u) return -1;
    for (uint64_t i = 0; i < n; i++) u[i].key = k[i], u[i].val = v[i];
    int rc = g_spread_all(g, u, n);
    free(u);
    return rc;
}

/* init_csr_gpma (gpma.cuh:836-847): the V sentinels (value 1) and init_gpma's
 * two KEY_MAX guards (value 1).  init_gpma leaves segment_length 32 over a
 * 4-slot array, so the reference's first update reads and writes past it
 * (gpma.cuh:185-187, 229-231); here the first state is the one that
 * update's resize path gives: everything spread over the smallest power of
 * two >= V + 2. */
OGpma *ogpma_create(uint32_t V, double density_lower) {
    if (V == 0 || V >= 0xFFFFFFFFu) return NULL;
    OGpma *g = (OGpma *)calloc(1, sizeof(OGpma));
    if (!g) return NULL;
    g->V = V;
    g->dlow = density_lower;
    g->row = (uint32_t *)calloc((size_t)V + 1, sizeof(uint32_t));
    g->size = 4;
    g->keys = (uint64_t *)malloc(4 * sizeof(uint64_t));
    g->vals = (uint8_t *)calloc(4, 1);
    if (!g->row || !g->keys || !g->vals) return NULL;
    for (int i = 0; i < 4; i++) g->keys[i] = KEY_NONE;
    g->seg = 2;
    g->h = 1;
    uint64_t *k = (uint64_t *)malloc(((size_t)V + 2) * sizeof(uint64_t));
    uint8_t *v = (uint8_t *)malloc((size_t)V + 2);
    for (uint32_t i = 0; i < V; i++) k[i] = ((uint64_t)i << 32) | G_COL_NONE, v[i] = 1;
    k[V] = k[V + 1] = G_KEY_MAX;
    v[V] = v[V + 1] = 1;
    int rc = g_build_from(g, k, v, (uint64_t)V + 2);
    free(k);
    free(v);
    if (rc) return NULL;
    return g;
}

void ogpma_destroy(OGpma *g) {
    if (!g) return;
    free(g->keys);
    free(g->vals);
    free(g->row);
    free(g);
}

/* update_gpma (gpma.cuh:747-816) for a batch of inserts (values ins_vals or
 * 1) and deletes (updates with VALUE_NONE).  Extension, as for the leveled
 * array: the batch is resolved to a set first (an insert and a delete of one
 * key apply delete-first, the last insert of a key gives its value); the
 * reference applies repeated keys of one batch from concurrent threads. */
int ogpma_update(OGpma *g, const uint64_t *ins, const uint8_t *ins_vals, size_t n_ins, const uint64_t *del,
                 size_t n_del, OPmaStats *st) {
    OPmaStats dummy;
    if (!st) st = &dummy;
    memset(st, 0, sizeof(*st));
    st->height_before = g->h;
    size_t n = n_ins + n_del;
    for (size_t i = 0; i < n_ins; i++) {
        if ((ins[i] >> 32) >= g->V || (ins[i] & G_COL_NONE) >= g->V) return -2;
        if (ins_vals && ins_vals[i] == VAL_TOMB) return -2;
    }
    for (size_t i = 0; i < n_del; i++)
        if ((del[i] >> 32) >= g->V || (del[i] & G_COL_NONE) >= g->V) return -2;
    if (n == 0) {
        st->height_after = g->h;
        return 0;
    }
    Ent *e = (Ent *)malloc(n * sizeof(Ent));
    Upd *u = (Upd *)malloc(n * sizeof(Upd));
    if (!e || !u) return -1;
    for (size_t i = 0; i < n_ins; i++) e[i] = (Ent){ins[i], (uint32_t)i, K_INS, ins_vals ? ins_vals[i] : (uint8_t)1};
    for (size_t i = 0; i < n_del; i++) e[n_ins + i] = (Ent){del[i], (uint32_t)(n_ins + i), K_DEL, 0};
    qsort(e, n, sizeof(Ent), cmp_ent);
    size_t np = 0;
    for (size_t i = 0; i < n;) {
        size_t j = i;
        while (j < n && e[j].key == e[i].key) j++;
        const Ent *rep = &e[i];
        if (e[i].kind == K_INS) {
            size_t q = i;
            while (q + 1 < j && e[q + 1].kind == K_INS) q++;
            rep = &e[q];
        }
        st->n_noop += (uint32_t)(j - i - 1);
        /* locate + handle_del_mod: the first equal key of the segment */
        const uint64_t node = g_locate(g, rep->key);
        int64_t hit = -1;
        for (uint32_t l = 0; l < g->seg; l++)
            if (g->keys[node + l] == rep->key) {
                hit = (int64_t)(node + l);
                break;
            }
        if (rep->kind == K_INS) {
            if (hit >= 0) {
                if (g->vals[hit] == VAL_TOMB)
                    st->n_ins_applied++; /* a tombstoned key comes back in place */
                else
                    st->n_upserts++;
                g->vals[hit] = rep->val;
            } else {
                u[np] = (Upd){rep->key, node, rep->val, K_INS, 0};
                np++;
                st->n_ins_applied++;
            }
        } else {
            if (hit >= 0 && g->vals[hit] != VAL_TOMB) {
                g->vals[hit] = VAL_TOMB;
                st->n_del_applied++;
            } else {
                st->n_noop++;
            }
        }
        i = j;
    }
    free(e);
    int rc = 0;
    if (np >= G_SIGNIFICANT) {
        /* significant_insert, gpma.cuh:771-776 */
        st->rebuilt = 1;
        st->levelup = 1;
        rc = g_spread_all(g, u, np);
        np = 0;
    }
    GItem *buf = (GItem *)malloc((g->size + np + 1) * sizeof(GItem));
    uint64_t *mk = (uint64_t *)malloc((g->size + np + 1) * sizeof(uint64_t));
    uint8_t *mv = (uint8_t *)malloc(g->size + np + 1);
    if (!buf || !mk || !mv) return -1;
    /* the level loop, gpma.cuh:779-797 */
    for (uint32_t level = 0; level <= g->h && np > 0 && rc == 0; level++) {
        const uint64_t width = (uint64_t)g->seg << level;
        const uint32_t lower = g->lower[level], upper = g->upper[level];
        for (size_t i = 0; i < np;) {
            size_t j = i;
            const uint64_t node = u[i].node;
            while (j < np && u[j].node == node) j++;
            /* compaction: in place for windows of up to 1024 slots
             * (block_compact_kernel, whatever the check decides), into
             * scratch above (compact_kernel) */
            uint64_t c = 0;
            for (uint64_t q = 0; q < width; q++)
                if (g_kept(g->keys[node + q], g->vals[node + q])) {
                    buf[c] = (GItem){g->keys[node + q], c, g->vals[node + q]};
                    c++;
                }
            if (width <= 1024) {
                for (uint64_t q = 0; q < width; q++) g->keys[node + q] = KEY_NONE;
                for (uint64_t q = 0; q < c; q++) g->keys[node + q] = buf[q].key, g->vals[node + q] = buf[q].val;
            }
            const uint64_t m = c + (j - i);
            if (lower <= m && m <= upper) {
                for (size_t q = i; q < j; q++) {
                    buf[c + (q - i)] = (GItem){u[q].key, c + (q - i), u[q].val};
                    u[q].applied = 1;
                }
                g_merge_sorted(buf, m, mk, mv);
                g_spread(g, mk, mv, m, node, width);
                if (level < 32) {
                    st->win_count[level]++;
                    st->win_slots[level] += width;
                }
                if (level == g->h) st->root_executed = 1;
            }
            i = j;
        }
        size_t o = 0;
        for (size_t q = 0; q < np; q++)
            if (!u[q].applied) {
                u[o] = u[q];
                u[o].node &= ~width;
                o++;
            }
        np = o;
    }
    free(buf);
    free(mk);
    free(mv);
    if (np > 0 && rc == 0) {
        /* the root could not take them: resize_gpma + root rebalance,
         * gpma.cuh:800-813 */
        st->overflow = 1;
        st->rebuilt = 1;
        st->root_executed = 1;
        st->levelup = 1;
        rc = g_spread_all(g, u, np);
    }
    free(u);
    st->height_after = g->h;
    return rc;
}

uint64_t ogpma_size(const OGpma *g, uint32_t *seg, uint32_t *h) {
    if (seg) *seg = g->seg;
    if (h) *h = g->h;
    return g->size;
}

/* the flat array (empty slots: key ~0, value 0) and row_offset */
int ogpma_layout(const OGpma *g, uint64_t *keys, uint8_t *vals, size_t cap, uint32_t *row_offset) {
    if (cap < g->size) return -1;
    for (uint64_t i = 0; i < g->size; i++) {
        keys[i] = g->keys[i];
        vals[i] = g->keys[i] == KEY_NONE ? 0 : g->vals[i];
    }
    if (row_offset) memcpy(row_offset, g->row, ((size_t)g->V + 1) * sizeof(uint32_t));
    return 0;
}

/* live keys (tombstones and the two guards left out), sorted */
int64_t ogpma_export_sorted(const OGpma *g, uint64_t *keys, uint8_t *vals, size_t cap) {
    int64_t o = 0;
    for (uint64_t i = 0; i < g->size; i++)
        if (g_kept(g->keys[i], g->vals[i]) && g->keys[i] != G_KEY_MAX) {
            if ((size_t)o >= cap) return -1;
            keys[o] = g->keys[i];
            if (vals) vals[o] = g->vals[i];
            o++;
        }
    return o;
}

/* test hooks for the comparison with the reference's compiled functions */
void ogpma_size_rule(uint64_t merge, uint64_t *size, uint32_t *seg, uint32_t *h) { g_size_rule(merge, size, seg, h); }
void ogpma_density(uint32_t seg, uint32_t h, double dlow, uint32_t *lower, uint32_t *upper) {
    OGpma t;
    memset(&t, 0, sizeof(t));
    t.seg = seg;
    t.h = h;
    t.dlow = dlow;
    g_density(&t);
    for (uint32_t i = 0; i <= h && i < 40; i++) lower[i] = t.lower[i], upper[i] = t.upper[i];
}
/* locate + handle_del_mod alone, literally, for n updates in order (value
 * VALUE_NONE: delete): leaf[i] = the located slot, or 0xFFFFFFFF when the
 * update was applied in place or is a delete (gpma.cuh:162-200) */
int ogpma_resolve_only(OGpma *g, const uint64_t *keys, const uint8_t *vals, size_t n, uint32_t *leaf) {
    for (size_t i = 0; i < n; i++) {
        uint64_t node = g_locate(g, keys[i]);
        uint32_t lf = vals[i] == VAL_TOMB ? 0xFFFFFFFFu : (uint32_t)node;
        for (uint32_t l = 0; l < g->seg; l++)
            if (g->keys[node + l] == keys[i]) {
                g->vals[node + l] = vals[i];
                lf = 0xFFFFFFFFu;
                break;
            }
        leaf[i] = lf;
    }
    return 0;
}

/* g_spread over [node, node + width) of a caller's flat array */
int ogpma_spread_window(uint32_t V, uint32_t seg, uint64_t node, uint64_t width, const uint64_t *mk, const uint8_t *mv,
                        uint64_t m, uint64_t *keys, uint8_t *vals, uint32_t *row_offset) {
    OGpma t;
    memset(&t, 0, sizeof(t));
    t.V = V;
    t.seg = seg;
    t.keys = keys;
    t.vals = vals;
    t.row = row_offset;
    if (m > width) return -1;
    g_spread(&t, mk, mv, m, node, width);
    return 0;
}

int ogpma_locate_keys(const OGpma *g, const uint64_t *keys, size_t n, uint32_t *out) {
    for (size_t i = 0; i < n; i++) out[i] = (uint32_t)g_locate(g, keys[i]);
    return 0;
}

/* ------------------------------------------------------------------ */
/* CPU baseline: sorted-merge CSR rebuild per batch (test_cusparse.cu:51-78
 * sort-then-coo2csr method, test_algos.cu:197-203 host CSR build)        */
/* ------------------------------------------------------------------ */
struct OCsr {
    uint32_t V;
    int threads;
    uint64_t n, cap;
    uint64_t *e;   /* sorted edge keys */
    uint64_t *tmp; /* merge target */
    uint32_t *row; /* V+1: row_offset[v] = first edge of v */
};

OCsr *ocsr_create(uint32_t V, int threads) {
    OCsr *c = (OCsr *)calloc(1, sizeof(OCsr));
    c->V = V;
    c->threads = threads < 1 ? 1 : threads;
    c->row = (uint32_t *)calloc((size_t)V + 1, sizeof(uint32_t));
    return c;
}

void ocsr_destroy(OCsr *c) {
    if (!c) return;
    free(c->e);
    free(c->tmp);
    free(c->row);
    free(c);
}

static int ocsr_reserve(OCsr *c, uint64_t n) {
    if (n <= c->cap) return 0;
    uint64_t cap = n + n / 4 + 1024;
    uint64_t *e = (uint64_t *)realloc(c->e, cap * sizeof(uint64_t));
    uint64_t *t = (uint64_t *)realloc(c->tmp, cap * sizeof(uint64_t));
    if (!e || !t) return -1;
    c->e = e;
    c->tmp = t;
    c->cap = cap;
    return 0;
}

typedef struct {
    const uint64_t *a, *b;
    uint64_t a0, a1, b0, b1; /* this worker's key-range partition */
    uint64_t *out;
    int subtract;
    uint64_t written;
    OCsr *c;
    uint32_t v0, v1;
} MergeJob;

static uint64_t lower_bound_u64(const uint64_t *x, uint64_t n, uint64_t key) {
    uint64_t lo = 0, hi = n;
    while (lo < hi) {
        uint64_t mid = (lo + hi) >> 1;
        if (x[mid] < key)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

static void *merge_worker(void *arg) {
    MergeJob *j = (MergeJob *)arg;
    uint64_t ia = j->a0, ib = j->b0, o = 0;
    if (!j->subtract) {
        while (ia < j->a1 || ib < j->b1) {
            if (ib >= j->b1 || (ia < j->a1 && j->a[ia] <= j->b[ib])) {
                if (ib < j->b1 && j->a[ia] == j->b[ib]) ib++; /* key already present */
                j->out[o++] = j->a[ia++];
            } else
                j->out[o++] = j->b[ib++];
        }
    } else {
        while (ia < j->a1) {
            while (ib < j->b1 && j->b[ib] < j->a[ia]) ib++;
            if (ib < j->b1 && j->b[ib] == j->a[ia]) {
                ia++;
                ib++;
            } else
                j->out[o++] = j->a[ia++];
        }
    }
    j->written = o;
    return NULL;
}

static void *row_worker(void *arg) {
    MergeJob *j = (MergeJob *)arg;
    OCsr *c = j->c;
    for (uint32_t v = j->v0; v < j->v1; v++) c->row[v] = (uint32_t)lower_bound_u64(c->e, c->n, (uint64_t)v << SRC_SHIFT);
    return NULL;
}

static int ocsr_apply(OCsr *c, const uint64_t *keys, uint64_t n, int subtract) {
    uint64_t *b = (uint64_t *)malloc((n ? n : 1) * sizeof(uint64_t));
    if (!b) return -1;
    memcpy(b, keys, n * sizeof(uint64_t));
    radix_sort_u64(b, NULL, n);
    uint64_t w = 0;
    for (uint64_t i = 0; i < n; i++)
        if (w == 0 || b[w - 1] != b[i]) b[w++] = b[i];
    n = w;
    if (ocsr_reserve(c, c->n + n)) return -1;
    int T = c->threads > 256 ? 256 : c->threads;
    uint64_t big = c->n > n ? c->n : n;
    if ((uint64_t)T > big / 64 + 1) T = (int)(big / 64 + 1);
    MergeJob jobs[256];
    pthread_t th[256];
    const uint64_t *sx = c->n >= n ? c->e : b; /* splitters from the larger input */
    uint64_t sn = big;
    for (int t = 0; t < T; t++) {
        uint64_t k0 = t == 0 ? 0 : sx[sn * t / T];
        uint64_t k1 = t == T - 1 ? 0 : sx[sn * (t + 1) / T];
        jobs[t].a = c->e;
        jobs[t].b = b;
        jobs[t].a0 = t == 0 ? 0 : lower_bound_u64(c->e, c->n, k0);
        jobs[t].b0 = t == 0 ? 0 : lower_bound_u64(b, n, k0);
        jobs[t].a1 = t == T - 1 ? c->n : lower_bound_u64(c->e, c->n, k1);
        jobs[t].b1 = t == T - 1 ? n : lower_bound_u64(b, n, k1);
        jobs[t].subtract = subtract;
        jobs[t].out = c->tmp + jobs[t].a0 + jobs[t].b0;
        jobs[t].c = c;
    }
    for (int t = 0; t < T; t++) {
        if (T > 1)
            pthread_create(&th[t], NULL, merge_worker, &jobs[t]);
        else
            merge_worker(&jobs[t]);
    }
    if (T > 1)
        for (int t = 0; t < T; t++) pthread_join(th[t], NULL);
    /* close the gaps left by duplicate or removed keys */
    uint64_t o = 0;
    for (int t = 0; t < T; t++) {
        uint64_t from = jobs[t].a0 + jobs[t].b0;
        if (from != o) memmove(c->tmp + o, c->tmp + from, jobs[t].written * sizeof(uint64_t));
        o += jobs[t].written;
    }
    uint64_t *sw = c->e;
    c->e = c->tmp;
    c->tmp = sw;
    c->n = o;
    /* row_offset rebuild */
    int TR = c->threads > 256 ? 256 : c->threads;
    if ((uint32_t)TR > c->V) TR = 1;
    for (int t = 0; t < TR; t++) {
        jobs[t].v0 = (uint32_t)((uint64_t)c->V * t / TR);
        jobs[t].v1 = (uint32_t)((uint64_t)c->V * (t + 1) / TR);
        jobs[t].c = c;
        if (TR > 1)
            pthread_create(&th[t], NULL, row_worker, &jobs[t]);
        else
            row_worker(&jobs[t]);
    }
    if (TR > 1)
        for (int t = 0; t < TR; t++) pthread_join(th[t], NULL);
    c->row[c->V] = (uint32_t)c->n;
    free(b);
    return 0;
}

int ocsr_load(OCsr *c, const uint64_t *keys, uint64_t n) {
    c->n = 0;
    return ocsr_apply(c, keys, n, 0);
}
int ocsr_insert(OCsr *c, const uint64_t *keys, uint64_t n) { return ocsr_apply(c, keys, n, 0); }
int ocsr_delete(OCsr *c, const uint64_t *keys, uint64_t n) { return ocsr_apply(c, keys, n, 1); }
uint64_t ocsr_num_edges(const OCsr *c) { return c->n; }
const uint64_t *ocsr_edges(const OCsr *c) { return c->e; }
const uint32_t *ocsr_row_offset(const OCsr *c) { return c->row; }
