/*
 * fhe_oracle.c — CPU restatement of PhantomFHE's RNS ciphertext arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY: this is the checker used by tests/, by the smoke check and
 * by bench.py's CPU-baseline leg.  It is never linked into the GPU library.
 *
 * Every routine restates the reference function cited in fhe_oracle.h with plain loops,
 * unsigned __int128 arithmetic and exact reductions ("x % q"), so every result is the
 * canonical residue of the mathematically defined value.  The reference's FP64 steps
 * (BFV HPS base conversion and scale-and-round) are reproduced with explicit fma() in
 * the reference loop order, because nvcc contracts `acc += a * b` into a fused
 * multiply-add; this file must be compiled with -ffp-contract=off so the host compiler
 * does not fuse anything else.
 */
#include "fhe_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;

#define MAXP 96

/* ------------------------------------------------------------------ number theory */

uint64_t orc_mulmod(uint64_t a, uint64_t b, uint64_t q) { return (uint64_t)(((u128)a * b) % q); }

uint64_t orc_powmod(uint64_t a, uint64_t e, uint64_t q) {
    uint64_t r = 1 % q;
    a %= q;
    while (e) {
        if (e & 1) r = orc_mulmod(r, a, q);
        a = orc_mulmod(a, a, q);
        e >>= 1;
    }
    return r;
}

/* Extended Euclid (xgcd in include/host/numth.h). Returns 0 when not invertible. */
uint64_t orc_invmod(uint64_t a, uint64_t q) {
    a %= q;
    if (a == 0) return 0;
    __int128 t0 = 0, t1 = 1;
    __int128 r0 = q, r1 = a;
    while (r1 != 0) {
        __int128 qq = r0 / r1, tmp;
        tmp = r0 - qq * r1; r0 = r1; r1 = tmp;
        tmp = t0 - qq * t1; t0 = t1; t1 = tmp;
    }
    if (r0 != 1) return 0;
    if (t0 < 0) t0 += q;
    return (uint64_t)t0;
}

/* Deterministic Miller-Rabin over the first 12 prime bases (exact for all 64-bit
 * inputs).  The reference (numth.cu:129-205) uses base 2 plus random bases: both accept
 * every prime, so the prime lists agree. */
int orc_is_prime(uint64_t v) {
    static const uint64_t small[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
    if (v < 2) return 0;
    for (int i = 0; i < 12; i++) {
        if (v == small[i]) return 1;
        if (v % small[i] == 0) return 0;
    }
    uint64_t d = v - 1;
    int r = 0;
    while ((d & 1) == 0) { d >>= 1; r++; }
    for (int i = 0; i < 12; i++) {
        uint64_t x = orc_powmod(small[i], d, v);
        if (x == 1 || x == v - 1) continue;
        int ok = 0;
        for (int k = 1; k < r; k++) {
            x = orc_mulmod(x, x, v);
            if (x == v - 1) { ok = 1; break; }
        }
        if (!ok) return 0;
    }
    return 1;
}

void orc_barrett_ratio(uint64_t q, uint64_t out[3]) {
    /* floor(2^128 / q) and 2^128 mod q, computed as 2^128 = (2^128 - 1) + 1. */
    u128 m = ~(u128)0;
    u128 quo = m / q;
    u128 rem = m % q;
    rem += 1;
    if (rem == q) { quo += 1; rem = 0; }
    out[0] = (uint64_t)quo;
    out[1] = (uint64_t)(quo >> 64);
    out[2] = (uint64_t)rem;
}

uint64_t orc_shoup(uint64_t w, uint64_t q) { return (uint64_t)(((u128)w << 64) / q); }

int orc_get_primes(uint64_t n, int bits, int count, uint64_t *out) {
    uint64_t factor = 2 * n;
    uint64_t value = ((uint64_t)1 << bits) - factor + 1;
    uint64_t lower = (uint64_t)1 << (bits - 1);
    int got = 0;
    while (got < count && value > lower) {
        if (orc_is_prime(value)) out[got++] = value;
        value -= factor;
    }
    return got == count ? 0 : -1;
}

static int sig_bits(uint64_t v) {
    int b = 0;
    while (v) { b++; v >>= 1; }
    return b;
}

int orc_get_primes_below(uint64_t n, uint64_t upper, int count, uint64_t *out) {
    uint64_t factor = 2 * n;
    uint64_t value = upper - factor;
    uint64_t lower = (uint64_t)1 << (sig_bits(upper) - 1);
    int got = 0;
    while (got < count && value > lower) {
        if (orc_is_prime(value)) out[got++] = value;
        value -= factor;
    }
    return got == count ? 0 : -1;
}

int orc_create_coeff_modulus(uint64_t n, const int *bit_sizes, int count, uint64_t *out) {
    /* For each distinct bit size, generate all the primes it needs (descending), then hand
     * them out from the back of the list in order of appearance. */
    int sizes[64], counts[64], used[64], nsz = 0;
    uint64_t lists[64][64];
    for (int i = 0; i < count; i++) {
        int k;
        for (k = 0; k < nsz; k++)
            if (sizes[k] == bit_sizes[i]) break;
        if (k == nsz) { sizes[nsz] = bit_sizes[i]; counts[nsz] = 0; used[nsz] = 0; nsz++; }
        counts[k]++;
    }
    for (int k = 0; k < nsz; k++)
        if (orc_get_primes(n, sizes[k], counts[k], lists[k])) return -1;
    for (int i = 0; i < count; i++) {
        int k;
        for (k = 0; k < nsz; k++)
            if (sizes[k] == bit_sizes[i]) break;
        out[i] = lists[k][counts[k] - 1 - used[k]];
        used[k]++;
    }
    return 0;
}

uint64_t orc_minimal_root(uint64_t degree, uint64_t q) {
    if ((q - 1) % degree) return 0;
    uint64_t quot = (q - 1) / degree, g = 0;
    for (uint64_t x = 2; x < q; x++) {
        g = orc_powmod(x, quot, q);
        if (orc_powmod(g, degree / 2, q) == q - 1) break;
    }
    /* Every primitive root is g^k with k odd; take the smallest (numth.cu:309-331). */
    uint64_t g2 = orc_mulmod(g, g, q), cur = g, best = g;
    for (uint64_t i = 0; i < degree / 2; i++) {
        if (cur < best) best = cur;
        cur = orc_mulmod(cur, g2, q);
    }
    return best;
}

static uint32_t bitrev(uint32_t x, int bits) {
    uint32_t r = 0;
    for (int i = 0; i < bits; i++) { r = (r << 1) | (x & 1); x >>= 1; }
    return r;
}

int orc_ntt_tables(int log_n, uint64_t q, uint64_t *root, uint64_t *root_shoup, uint64_t *inv_root,
                   uint64_t *inv_root_shoup, uint64_t *n_inv) {
    uint64_t n = (uint64_t)1 << log_n;
    uint64_t psi = orc_minimal_root(2 * n, q);
    if (!psi) return -1;
    uint64_t ipsi = orc_invmod(psi, q);
    uint64_t p = psi, ip = ipsi;
    root[0] = 1;
    inv_root[0] = 1;
    for (uint64_t i = 1; i < n; i++) {
        root[bitrev((uint32_t)i, log_n)] = p;
        inv_root[bitrev((uint32_t)i, log_n)] = ip;
        p = orc_mulmod(p, psi, q);
        ip = orc_mulmod(ip, ipsi, q);
    }
    uint64_t ni = orc_invmod(n, q);
    inv_root[1] = orc_mulmod(inv_root[1], ni, q);
    for (uint64_t i = 0; i < n; i++) {
        if (root_shoup) root_shoup[i] = orc_shoup(root[i], q);
        if (inv_root_shoup) inv_root_shoup[i] = orc_shoup(inv_root[i], q);
    }
    *n_inv = ni;
    return 0;
}

/* ------------------------------------------------------------------ context */

typedef struct {
    uint64_t q;
    uint64_t *root, *root_sh, *iroot, *iroot_sh;
    uint64_t n_inv, n_inv_sh;
} orc_tab;

struct orc_ctx {
    int log_n, n, nQ, nP, nR;
    uint64_t t;
    uint64_t mod[MAXP]; /* QP */
    orc_tab tab[MAXP];
    uint64_t rmod[MAXP]; /* HPS R base */
    orc_tab rtab[MAXP];
};

static int g_threads = 0;
void orc_set_threads(int threads) { g_threads = threads; }
#ifdef _OPENMP
#define OMP_THREADS (g_threads > 0 ? g_threads : omp_get_max_threads())
#endif

static int make_tab(orc_tab *t, int log_n, uint64_t q) {
    size_t n = (size_t)1 << log_n;
    t->q = q;
    t->root = malloc(n * 8); t->root_sh = malloc(n * 8);
    t->iroot = malloc(n * 8); t->iroot_sh = malloc(n * 8);
    if (orc_ntt_tables(log_n, q, t->root, t->root_sh, t->iroot, t->iroot_sh, &t->n_inv)) return -1;
    t->n_inv_sh = orc_shoup(t->n_inv, q);
    return 0;
}

static void free_tab(orc_tab *t) {
    free(t->root); free(t->root_sh); free(t->iroot); free(t->iroot_sh);
}

orc_ctx *orc_ctx_create(int log_n, const uint64_t *moduli, int nQ, int nP, uint64_t plain_modulus) {
    if (nQ + nP > MAXP || nQ < 1) return NULL;
    orc_ctx *c = calloc(1, sizeof(orc_ctx));
    c->log_n = log_n;
    c->n = 1 << log_n;
    c->nQ = nQ;
    c->nP = nP;
    c->t = plain_modulus;
    for (int i = 0; i < nQ + nP; i++) {
        c->mod[i] = moduli[i];
        if (make_tab(&c->tab[i], log_n, moduli[i])) { orc_ctx_destroy(c); return NULL; }
    }
    if (plain_modulus) {
        /* HPS R base: |Q|+1 primes below the smallest Q prime (rns.cu:690-694). */
        uint64_t minq = moduli[0];
        for (int i = 1; i < nQ; i++)
            if (moduli[i] < minq) minq = moduli[i];
        c->nR = nQ + 1;
        if (orc_get_primes_below((uint64_t)c->n, minq, c->nR, c->rmod)) { orc_ctx_destroy(c); return NULL; }
        for (int j = 0; j < c->nR; j++)
            if (make_tab(&c->rtab[j], log_n, c->rmod[j])) { orc_ctx_destroy(c); return NULL; }
    }
    return c;
}

void orc_ctx_destroy(orc_ctx *c) {
    if (!c) return;
    for (int i = 0; i < c->nQ + c->nP; i++)
        if (c->tab[i].root) free_tab(&c->tab[i]);
    for (int j = 0; j < c->nR; j++)
        if (c->rtab[j].root) free_tab(&c->rtab[j]);
    free(c);
}

int orc_ctx_n(const orc_ctx *c) { return c->n; }

int orc_ctx_hps_r(const orc_ctx *c, uint64_t *r_out) {
    if (r_out)
        for (int j = 0; j < c->nR; j++) r_out[j] = c->rmod[j];
    return c->nR;
}

/* ------------------------------------------------------------------ NTT */

static inline uint64_t mul_shoup(uint64_t x, uint64_t w, uint64_t w_sh, uint64_t q) {
    uint64_t hi = (uint64_t)(((u128)x * w_sh) >> 64);
    uint64_t r = x * w - hi * q;
    return r >= q ? r - q : r;
}

/* Forward negacyclic NTT, Cooley-Tukey, bit-reversed powers (the transform computed by
 * nwt_2d_radix8_forward_inplace, src/ntt/fntt_2d.cu:620-653). */
static void ntt_fwd_one(uint64_t *a, const orc_tab *t, int n) {
    const uint64_t q = t->q;
    for (int m = 1, h = n >> 1; m < n; m <<= 1, h >>= 1) {
        for (int i = 0; i < m; i++) {
            uint64_t w = t->root[m + i], ws = t->root_sh[m + i];
            uint64_t *x = a + 2 * i * h, *y = x + h;
            for (int j = 0; j < h; j++) {
                uint64_t u = x[j], v = mul_shoup(y[j], w, ws, q);
                uint64_t s = u + v;
                x[j] = s >= q ? s - q : s;
                y[j] = u >= v ? u - v : u + q - v;
            }
        }
    }
}

/* Inverse transform, Gentleman-Sande, with n^-1 folded into inv_root[1] for the last stage
 * (nwt_2d_radix8_backward_inplace, src/ntt/intt_2d.cu:724-757, tables src/host/ntt.cu:53-55). */
static void ntt_inv_one(uint64_t *a, const orc_tab *t, int n) {
    const uint64_t q = t->q;
    for (int m = n >> 1, h = 1; m >= 1; m >>= 1, h <<= 1) {
        for (int i = 0; i < m; i++) {
            uint64_t w = t->iroot[m + i], ws = t->iroot_sh[m + i];
            uint64_t *x = a + 2 * i * h, *y = x + h;
            for (int j = 0; j < h; j++) {
                uint64_t u = x[j], v = y[j];
                uint64_t s = u + v;
                s = s >= q ? s - q : s;
                uint64_t d = u >= v ? u - v : u + q - v;
                if (m == 1) s = mul_shoup(s, t->n_inv, t->n_inv_sh, q);
                x[j] = s;
                y[j] = mul_shoup(d, w, ws, q);
            }
        }
    }
}

void orc_ntt_fwd(const orc_ctx *c, uint64_t *data, int num_limbs, const int *tbl) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(OMP_THREADS)
    for (int k = 0; k < num_limbs; k++)
        ntt_fwd_one(data + (size_t)k * c->n, &c->tab[tbl ? tbl[k] : k], c->n);
}

void orc_ntt_inv(const orc_ctx *c, uint64_t *data, int num_limbs, const int *tbl) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(OMP_THREADS)
    for (int k = 0; k < num_limbs; k++)
        ntt_inv_one(data + (size_t)k * c->n, &c->tab[tbl ? tbl[k] : k], c->n);
}

static const orc_tab *qr_tab(const orc_ctx *c, int k) { return k < c->nQ ? &c->tab[k] : &c->rtab[k - c->nQ]; }

void orc_ntt_fwd_qr(const orc_ctx *c, uint64_t *data, int num_limbs) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(OMP_THREADS)
    for (int k = 0; k < num_limbs; k++) ntt_fwd_one(data + (size_t)k * c->n, qr_tab(c, k), c->n);
}

void orc_ntt_inv_qr(const orc_ctx *c, uint64_t *data, int num_limbs) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(OMP_THREADS)
    for (int k = 0; k < num_limbs; k++) ntt_inv_one(data + (size_t)k * c->n, qr_tab(c, k), c->n);
}

/* ------------------------------------------------------------------ element-wise */

static void tensor_limbs(const uint64_t *mods, int limbs, int n, const uint64_t *a, const uint64_t *b,
                         uint64_t *out) {
    size_t ln = (size_t)limbs * n;
#pragma omp parallel for num_threads(OMP_THREADS)
    for (int k = 0; k < limbs; k++) {
        uint64_t q = mods[k];
        for (int c = 0; c < n; c++) {
            size_t i = (size_t)k * n + c;
            uint64_t a0 = a[i], a1 = a[i + ln], b0 = b[i], b1 = b[i + ln];
            uint64_t d0 = orc_mulmod(a0, b0, q);
            uint64_t d2 = orc_mulmod(a1, b1, q);
            uint64_t d1 = (uint64_t)(((u128)a0 * b1 + (u128)a1 * b0) % q);
            out[i] = d0;
            out[i + ln] = d1;
            out[i + 2 * ln] = d2;
        }
    }
}

void orc_tensor(const orc_ctx *c, int l, const uint64_t *a, const uint64_t *b, uint64_t *out3) {
    tensor_limbs(c->mod, l, c->n, a, b, out3);
}

void orc_tensor_square(const orc_ctx *c, int l, const uint64_t *a, uint64_t *out3) {
    tensor_limbs(c->mod, l, c->n, a, a, out3);
}

/* ------------------------------------------------------------------ key switching */

/* QlP limb index -> QP table index (include_special_mod remap, src/ntt/ntt_modup.cu:423-425). */
static int qlp_index(const orc_ctx *c, int l, int jj) { return jj < l ? jj : c->nQ + (jj - l); }

/* prod_{k in [s, s+sz), k != skip} mods[k] mod p */
static uint64_t prod_except_mod(const uint64_t *mods, int s, int sz, int skip, uint64_t p) {
    uint64_t r = 1 % p;
    for (int k = s; k < s + sz; k++)
        if (k != skip) r = orc_mulmod(r, mods[k] % p, p);
    return r;
}

int orc_modup_tables(const orc_ctx *c, int l, int d, uint64_t *part_hat_inv, uint64_t *matrix) {
    int alpha = c->nP, s = d * alpha;
    if (s >= l) return -1;
    int sz = (l - s) < alpha ? (l - s) : alpha;
    for (int i = 0; i < sz; i++) {
        uint64_t q = c->mod[s + i];
        part_hat_inv[i] = orc_invmod(prod_except_mod(c->mod, s, sz, s + i, q), q);
    }
    int row = 0;
    for (int jj = 0; jj < l + c->nP; jj++) {
        if (jj >= s && jj < s + sz) continue;
        uint64_t p = c->mod[qlp_index(c, l, jj)];
        for (int i = 0; i < sz; i++) matrix[row * sz + i] = prod_except_mod(c->mod, s, sz, s + i, p);
        row++;
    }
    return sz;
}

void orc_modup(const orc_ctx *c, int l, const uint64_t *c2, uint64_t *out, int scheme) {
    const int n = c->n, alpha = c->nP, qlp = l + alpha;
    const int beta = (l + alpha - 1) / alpha;
    uint64_t *y = malloc((size_t)l * n * 8);
    memcpy(y, c2, (size_t)l * n * 8);
    if (scheme == 0) orc_ntt_inv(c, y, l, NULL); /* CKKS: back to coefficients */
    for (int d = 0; d < beta; d++) {
        int s = d * alpha, sz = (l - s) < alpha ? (l - s) : alpha;
        uint64_t phi[MAXP];
        for (int i = 0; i < sz; i++) {
            uint64_t q = c->mod[s + i];
            phi[i] = orc_invmod(prod_except_mod(c->mod, s, sz, s + i, q), q);
        }
        uint64_t *od = out + (size_t)d * qlp * n;
        int tbl[MAXP];
        int ntbl = 0;
        uint64_t *ydig = malloc((size_t)sz * n * 8);
        for (int i = 0; i < sz; i++) {
            uint64_t q = c->mod[s + i], ph = phi[i], phs = orc_shoup(phi[i], q);
            for (int k = 0; k < n; k++) ydig[(size_t)i * n + k] = mul_shoup(y[(size_t)(s + i) * n + k], ph, phs, q);
        }
#pragma omp parallel for schedule(dynamic, 1) num_threads(OMP_THREADS)
        for (int jj = 0; jj < qlp; jj++) {
            uint64_t *dst = od + (size_t)jj * n;
            if (jj >= s && jj < s + sz) {
                memcpy(dst, c2 + (size_t)jj * n, (size_t)n * 8);
                if (scheme == 1) ntt_fwd_one(dst, &c->tab[jj], n);
                continue;
            }
            int ti = qlp_index(c, l, jj);
            uint64_t p = c->mod[ti];
            uint64_t m[MAXP];
            for (int i = 0; i < sz; i++) m[i] = prod_except_mod(c->mod, s, sz, s + i, p);
            for (int k = 0; k < n; k++) {
                u128 acc = 0;
                for (int i = 0; i < sz; i++) acc += (u128)ydig[(size_t)i * n + k] * m[i];
                dst[k] = (uint64_t)(acc % p);
            }
            ntt_fwd_one(dst, &c->tab[ti], n);
        }
        (void)tbl; (void)ntbl;
        free(ydig);
    }
    free(y);
}

void orc_inner_product(const orc_ctx *c, int l, const uint64_t *tm, const uint64_t *evk, uint64_t *out) {
    const int n = c->n, alpha = c->nP, qlp = l + alpha, qp = c->nQ + c->nP;
    const int beta = (l + alpha - 1) / alpha;
#pragma omp parallel for schedule(dynamic, 1) num_threads(OMP_THREADS)
    for (int jj = 0; jj < qlp; jj++) {
        int ti = qlp_index(c, l, jj);
        uint64_t p = c->mod[ti];
        for (int k = 0; k < n; k++) {
            u128 a0 = 0, a1 = 0;
            for (int d = 0; d < beta; d++) {
                uint64_t x = tm[((size_t)d * qlp + jj) * n + k];
                const uint64_t *key = evk + (size_t)d * 2 * qp * n;
                a0 += (u128)x * key[(size_t)ti * n + k];
                a1 += (u128)x * key[((size_t)qp + ti) * n + k];
            }
            out[(size_t)jj * n + k] = (uint64_t)(a0 % p);
            out[((size_t)qlp + jj) * n + k] = (uint64_t)(a1 % p);
        }
    }
}

int orc_moddown_tables(const orc_ctx *c, int l, uint64_t *p_hat_inv, uint64_t *matrix, uint64_t *p_inv) {
    const int nP = c->nP, nQ = c->nQ;
    for (int k = 0; k < nP; k++) {
        uint64_t p = c->mod[nQ + k];
        p_hat_inv[k] = orc_invmod(prod_except_mod(c->mod, nQ, nP, nQ + k, p), p);
    }
    for (int j = 0; j < l; j++) {
        uint64_t q = c->mod[j];
        for (int k = 0; k < nP; k++) matrix[j * nP + k] = prod_except_mod(c->mod, nQ, nP, nQ + k, q);
        p_inv[j] = orc_invmod(prod_except_mod(c->mod, nQ, nP, -1, q), q);
    }
    return 0;
}

void orc_moddown(const orc_ctx *c, int l, uint64_t *cx, uint64_t *out, int scheme) {
    const int n = c->n, nP = c->nP, nQ = c->nQ;
    int tbl[MAXP];
    for (int jj = 0; jj < l + nP; jj++) tbl[jj] = qlp_index(c, l, jj);
    if (scheme == 0)
        orc_ntt_inv(c, cx + (size_t)l * n, nP, tbl + l);
    else
        orc_ntt_inv(c, cx, l + nP, tbl);
    uint64_t phinv[MAXP], mat[MAXP * MAXP], pinv[MAXP];
    orc_moddown_tables(c, l, phinv, mat, pinv);
    uint64_t *y = malloc((size_t)nP * n * 8);
    for (int k = 0; k < nP; k++) {
        uint64_t p = c->mod[nQ + k], s = orc_shoup(phinv[k], p);
        for (int i = 0; i < n; i++) y[(size_t)k * n + i] = mul_shoup(cx[(size_t)(l + k) * n + i], phinv[k], s, p);
    }
#pragma omp parallel for schedule(dynamic, 1) num_threads(OMP_THREADS)
    for (int j = 0; j < l; j++) {
        uint64_t q = c->mod[j];
        uint64_t *delta = malloc((size_t)n * 8);
        for (int i = 0; i < n; i++) {
            u128 acc = 0;
            for (int k = 0; k < nP; k++) acc += (u128)y[(size_t)k * n + i] * mat[j * nP + k];
            delta[i] = (uint64_t)(acc % q);
        }
        if (scheme == 0) ntt_fwd_one(delta, &c->tab[j], n);
        uint64_t ps = orc_shoup(pinv[j], q);
        for (int i = 0; i < n; i++) {
            uint64_t x = cx[(size_t)j * n + i], dl = delta[i];
            uint64_t diff = x >= dl ? x - dl : x + q - dl;
            out[(size_t)j * n + i] = mul_shoup(diff, pinv[j], ps, q);
        }
        free(delta);
    }
    free(y);
}

static void add_limbs(const uint64_t *mods, int limbs, int n, uint64_t *dst, const uint64_t *src) {
#pragma omp parallel for num_threads(OMP_THREADS)
    for (int k = 0; k < limbs; k++) {
        uint64_t q = mods[k];
        for (int i = 0; i < n; i++) {
            size_t x = (size_t)k * n + i;
            uint64_t s = dst[x] + src[x];
            dst[x] = s >= q ? s - q : s;
        }
    }
}

void orc_keyswitch(const orc_ctx *c, int l, uint64_t *ct, const uint64_t *c2, const uint64_t *evk, int scheme) {
    const int n = c->n, alpha = c->nP, qlp = l + alpha;
    const int beta = (l + alpha - 1) / alpha;
    uint64_t *tm = malloc((size_t)beta * qlp * n * 8);
    uint64_t *cx = malloc((size_t)2 * qlp * n * 8);
    uint64_t *md = malloc((size_t)l * n * 8);
    orc_modup(c, l, c2, tm, scheme);
    orc_inner_product(c, l, tm, evk, cx);
    for (int t = 0; t < 2; t++) {
        orc_moddown(c, l, cx + (size_t)t * qlp * n, md, scheme);
        add_limbs(c->mod, l, n, ct + (size_t)t * l * n, md);
    }
    free(tm); free(cx); free(md);
}

void orc_relinearize(const orc_ctx *c, int l, uint64_t *ct3, const uint64_t *rlk, int scheme) {
    orc_keyswitch(c, l, ct3, ct3 + (size_t)2 * l * c->n, rlk, scheme);
}

void orc_ckks_mul_relin(const orc_ctx *c, int l, const uint64_t *a, const uint64_t *b, const uint64_t *rlk,
                        uint64_t *out) {
    size_t ln = (size_t)l * c->n;
    uint64_t *t3 = malloc(3 * ln * 8);
    if (a == b)
        orc_tensor_square(c, l, a, t3);
    else
        orc_tensor(c, l, a, b, t3);
    orc_relinearize(c, l, t3, rlk, 0);
    memcpy(out, t3, 2 * ln * 8);
    free(t3);
}

void orc_rescale(const orc_ctx *c, int l, int size, const uint64_t *in, uint64_t *out) {
    const int n = c->n;
    uint64_t ql = c->mod[l - 1];
    for (int p = 0; p < size; p++) {
        const uint64_t *ci = in + (size_t)p * l * n;
        uint64_t *co = out + (size_t)p * (l - 1) * n;
        uint64_t *last = malloc((size_t)n * 8);
        memcpy(last, ci + (size_t)(l - 1) * n, (size_t)n * 8);
        ntt_inv_one(last, &c->tab[l - 1], n);
#pragma omp parallel for schedule(dynamic, 1) num_threads(OMP_THREADS)
        for (int j = 0; j < l - 1; j++) {
            uint64_t q = c->mod[j];
            uint64_t *dl = co + (size_t)j * n;
            for (int i = 0; i < n; i++) dl[i] = last[i] % q;
            ntt_fwd_one(dl, &c->tab[j], n);
            uint64_t inv = orc_invmod(ql % q, q), s = orc_shoup(inv, q);
            for (int i = 0; i < n; i++) {
                uint64_t x = ci[(size_t)j * n + i], d = dl[i];
                dl[i] = mul_shoup(x >= d ? x - d : x + q - d, inv, s, q);
            }
        }
        free(last);
    }
}

void orc_divide_round_q_last(const orc_ctx *c, int l, int size, const uint64_t *in, uint64_t *out) {
    const int n = c->n;
    uint64_t ql = c->mod[l - 1];
    for (int p = 0; p < size; p++) {
        const uint64_t *ci = in + (size_t)p * l * n;
        uint64_t *co = out + (size_t)p * (l - 1) * n;
        for (int j = 0; j < l - 1; j++) {
            uint64_t q = c->mod[j], inv = orc_invmod(ql % q, q);
            for (int i = 0; i < n; i++) {
                uint64_t x = ci[(size_t)j * n + i], d = ci[(size_t)(l - 1) * n + i] % q;
                co[(size_t)j * n + i] = orc_mulmod(x >= d ? x - d : x + q - d, inv, q);
            }
        }
    }
}

/* acc[p][k] += a[p][k] * b[k] mod q_k over `polys` polynomials of l limbs: the reference's
 * multiply_plain (multiply_rns_poly, src/polymath.cu) followed by add_inplace (add_rns_poly,
 * src/polymath.cu:41-55), as the matrix-vector inner sums use them
 * (python/src/binding.cu:545-566). */
void orc_mul_add(const orc_ctx *c, int l, int polys, const uint64_t *a, const uint64_t *b, uint64_t *acc) {
    const int n = c->n;
#pragma omp parallel for schedule(static) num_threads(OMP_THREADS)
    for (int pk = 0; pk < polys * l; pk++) {
        const int k = pk % l;
        const uint64_t q = c->mod[k];
        const uint64_t *ap = a + (size_t)pk * n, *bp = b + (size_t)k * n;
        uint64_t *cp = acc + (size_t)pk * n;
        for (int i = 0; i < n; i++) {
            uint64_t t = orc_mulmod(ap[i], bp[i], q) + cp[i];
            cp[i] = t >= q ? t - q : t;
        }
    }
}

/* ------------------------------------------------------------------ Galois */

uint32_t orc_elt_from_step(int step, uint64_t n) {
    uint32_t m32 = (uint32_t)(n * 2);
    uint64_t m = m32;
    if (step == 0) return (uint32_t)(m - 1);
    int sign = step < 0;
    uint32_t pos = (uint32_t)(step < 0 ? -step : step);
    if (pos >= (n >> 1)) return 0;
    pos &= m32 - 1;
    int s = sign ? (int)(n >> 1) - (int)pos : (int)pos;
    uint64_t elt = 1;
    while (s--) { elt *= 5; elt &= m - 1; }
    return (uint32_t)elt;
}

void orc_galois_perm(int log_n, uint32_t elt, uint32_t *perm) {
    uint32_t n = 1u << log_n;
    for (uint32_t i = n; i < 2 * n; i++) {
        uint32_t rev = bitrev(i, log_n + 1);
        uint64_t raw = ((uint64_t)elt * rev) >> 1;
        raw &= (uint64_t)(n - 1);
        perm[i - n] = bitrev((uint32_t)raw, log_n);
    }
}

void orc_apply_galois_ntt(const orc_ctx *c, const uint64_t *src, uint64_t *dst, int num_limbs, uint32_t elt) {
    const int n = c->n;
    uint32_t *perm = malloc((size_t)n * 4);
    orc_galois_perm(c->log_n, elt, perm);
    for (int k = 0; k < num_limbs; k++)
        for (int i = 0; i < n; i++) dst[(size_t)k * n + i] = src[(size_t)k * n + perm[i]];
    free(perm);
}

void orc_apply_galois_coeff(const orc_ctx *c, const uint64_t *src, uint64_t *dst, int num_limbs, uint32_t elt) {
    const uint64_t n = (uint64_t)c->n;
    for (int k = 0; k < num_limbs; k++) {
        uint64_t q = c->mod[k], raw = 0;
        for (uint64_t i = 0; i < n; i++) {
            uint64_t v = src[(size_t)k * n + i];
            if (raw >= n) v = v ? q - v : 0;
            dst[(size_t)k * n + (raw % n)] = v;
            raw = (raw + elt) & (2 * n - 1);
        }
    }
}

void orc_ckks_apply_galois(const orc_ctx *c, int l, uint64_t *ct, uint32_t elt, const uint64_t *gk) {
    size_t ln = (size_t)l * c->n;
    uint64_t *tmp = malloc(ln * 8);
    orc_apply_galois_ntt(c, ct, tmp, l, elt);
    memcpy(ct, tmp, ln * 8);
    orc_apply_galois_ntt(c, ct + ln, tmp, l, elt);
    memset(ct + ln, 0, ln * 8);
    orc_keyswitch(c, l, ct, tmp, gk, 0);
    free(tmp);
}

void orc_ckks_hoisting(const orc_ctx *c, int l, uint64_t *ct, const uint32_t *elts, int n_elts,
                       const uint64_t *const *gks) {
    const int n = c->n, alpha = c->nP, qlp = l + alpha;
    const int beta = (l + alpha - 1) / alpha;
    size_t ln = (size_t)l * n, qn = (size_t)qlp * n;
    uint64_t *acc0 = calloc(ln, 8), *tmp = malloc(ln * 8);
    uint64_t *mu = malloc(beta * qn * 8), *mup = malloc(beta * qn * 8);
    uint64_t *acc = calloc(2 * qn, 8), *cx = malloc(2 * qn * 8);
    uint64_t qlp_mods[MAXP];
    for (int jj = 0; jj < qlp; jj++) qlp_mods[jj] = c->mod[qlp_index(c, l, jj)];
    orc_modup(c, l, ct + ln, mu, 0);
    for (int s = 0; s < n_elts; s++) {
        orc_apply_galois_ntt(c, ct, tmp, l, elts[s]);
        add_limbs(c->mod, l, n, acc0, tmp);
        orc_apply_galois_ntt(c, mu, mup, beta * qlp, elts[s]);
        orc_inner_product(c, l, mup, gks[s], cx);
        add_limbs(qlp_mods, qlp, n, acc, cx);
        add_limbs(qlp_mods, qlp, n, acc + qn, cx + qn);
    }
    uint64_t *md = malloc(ln * 8);
    orc_moddown(c, l, acc, md, 0);
    add_limbs(c->mod, l, n, acc0, md);
    memcpy(ct, acc0, ln * 8);
    orc_moddown(c, l, acc + qn, md, 0);
    memcpy(ct + ln, md, ln * 8);
    free(acc0); free(tmp); free(mu); free(mup); free(acc); free(cx); free(md);
}

/* ------------------------------------------------------------------ BFV HPS */

/* Generic fast base conversion with the HPS FP64 correction (bconv_mult_unroll2_kernel +
 * base_convert_matmul_hps_unroll2_kernel, src/rns_bconv.cu:40-60, 310-352). */
static void hps_bconv(const uint64_t *ib, int ni, const uint64_t *ob, int no, int n, const uint64_t *in,
                      uint64_t *out) {
    uint64_t hinv[MAXP], m[MAXP][MAXP], qmod[MAXP];
    double qinv[MAXP];
    for (int i = 0; i < ni; i++) {
        hinv[i] = orc_invmod(prod_except_mod(ib, 0, ni, i, ib[i]), ib[i]);
        qinv[i] = 1.0 / (double)ib[i];
    }
    for (int j = 0; j < no; j++) {
        for (int i = 0; i < ni; i++) m[j][i] = prod_except_mod(ib, 0, ni, i, ob[j]);
        qmod[j] = prod_except_mod(ib, 0, ni, -1, ob[j]);
    }
#pragma omp parallel for num_threads(OMP_THREADS)
    for (int k = 0; k < n; k++) {
        uint64_t y[MAXP];
        double acc = 0.0;
        for (int i = 0; i < ni; i++) {
            y[i] = orc_mulmod(in[(size_t)i * n + k], hinv[i], ib[i]);
            acc = fma((double)y[i], qinv[i], acc);
        }
        uint64_t v = (uint64_t)llround(acc);
        for (int j = 0; j < no; j++) {
            u128 s = 0;
            for (int i = 0; i < ni; i++) s += (u128)y[i] * m[j][i];
            uint64_t r = (uint64_t)(s % ob[j]);
            uint64_t corr = orc_mulmod(v, qmod[j], ob[j]);
            out[(size_t)j * n + k] = r >= corr ? r - corr : r + ob[j] - corr;
        }
    }
}

void orc_hps_bconv_q_to_r(const orc_ctx *c, const uint64_t *in, uint64_t *out) {
    hps_bconv(c->mod, c->nQ, c->rmod, c->nR, c->n, in, out);
}

void orc_hps_bconv_r_to_q(const orc_ctx *c, const uint64_t *in, uint64_t *out) {
    hps_bconv(c->rmod, c->nR, c->mod, c->nQ, c->n, in, out);
}

int orc_hps_tables(const orc_ctx *c, double *frac, uint64_t *modr) {
    /* S = QR; for i in Q: X_i = t*R*[(S/s_i)^-1]_{s_i}, rem_i = X_i mod q_i,
     * frac_i = rem_i / q_i, and floor(X_i/q_i) mod r_j = -rem_i * q_i^-1 mod r_j (R | X_i).
     * For r_j itself: floor(X/r_j) = t*(R/r_j)*[(S/r_j)^-1]_{r_j}.  (rns.cu:714-777) */
    const int nQ = c->nQ, nR = c->nR;
    uint64_t s[2 * MAXP];
    for (int i = 0; i < nQ; i++) s[i] = c->mod[i];
    for (int j = 0; j < nR; j++) s[nQ + j] = c->rmod[j];
    for (int i = 0; i < nQ; i++) {
        uint64_t q = s[i];
        uint64_t shat_inv = orc_invmod(prod_except_mod(s, 0, nQ + nR, i, q), q);
        uint64_t r_mod_q = prod_except_mod(s, nQ, nR, -1, q);
        uint64_t rem = orc_mulmod(orc_mulmod(c->t % q, r_mod_q, q), shat_inv, q);
        frac[i] = (double)rem / (double)q;
        for (int j = 0; j < nR; j++) {
            uint64_t r = c->rmod[j];
            uint64_t v = orc_mulmod(rem % r, orc_invmod(q % r, r), r);
            modr[j * (nQ + 1) + i] = v ? r - v : 0;
        }
    }
    for (int j = 0; j < nR; j++) {
        uint64_t r = c->rmod[j];
        uint64_t shat_inv = orc_invmod(prod_except_mod(s, 0, nQ + nR, nQ + j, r), r);
        uint64_t rhat = prod_except_mod(s, nQ, nR, nQ + j, r);
        modr[j * (nQ + 1) + nQ] = orc_mulmod(orc_mulmod(c->t % r, rhat, r), shat_inv, r);
    }
    return 0;
}

void orc_hps_scale_round_qr_r(const orc_ctx *c, const uint64_t *in, uint64_t *out) {
    const int n = c->n, nQ = c->nQ, nR = c->nR;
    double frac[MAXP];
    uint64_t *modr = malloc((size_t)nR * (nQ + 1) * 8);
    orc_hps_tables(c, frac, modr);
#pragma omp parallel for num_threads(OMP_THREADS)
    for (int k = 0; k < n; k++) {
        double nu = 0.5;
        for (int i = 0; i < nQ; i++) nu = fma((double)in[(size_t)i * n + k], frac[i], nu);
        uint64_t alpha = (uint64_t)nu;
        for (int j = 0; j < nR; j++) {
            uint64_t r = c->rmod[j];
            u128 cur = 0;
            for (int i = 0; i < nQ; i++) cur += (u128)in[(size_t)i * n + k] * modr[j * (nQ + 1) + i];
            cur += (u128)in[(size_t)(nQ + j) * n + k] * modr[j * (nQ + 1) + nQ];
            uint64_t cv = (uint64_t)(cur % r);
            /* The reference reduces alpha in place, so r_j sees (alpha mod r_0 ...) mod r_j
             * (scaleAndRound_HPS_QR_R_kernel, src/rns.cu:1733). */
            alpha = alpha % r;
            uint64_t sum = cv + alpha;
            out[(size_t)j * n + k] = sum >= r ? sum - r : sum;
        }
    }
    free(modr);
}

void orc_bfv_mul_relin_hps(const orc_ctx *c, const uint64_t *a, const uint64_t *b, const uint64_t *rlk,
                           uint64_t *out) {
    const int n = c->n, nQ = c->nQ, nR = c->nR, qr = nQ + nR;
    size_t qn = (size_t)nQ * n, qrn = (size_t)qr * n;
    uint64_t *ea = malloc(2 * qrn * 8), *eb = malloc(2 * qrn * 8), *t3 = malloc(3 * qrn * 8);
    uint64_t s[2 * MAXP];
    for (int i = 0; i < nQ; i++) s[i] = c->mod[i];
    for (int j = 0; j < nR; j++) s[nQ + j] = c->rmod[j];
    for (int p = 0; p < 2; p++) {
        memcpy(ea + p * qrn, a + p * qn, qn * 8);
        orc_hps_bconv_q_to_r(c, a + p * qn, ea + p * qrn + qn);
        memcpy(eb + p * qrn, b + p * qn, qn * 8);
        orc_hps_bconv_q_to_r(c, b + p * qn, eb + p * qrn + qn);
    }
    orc_ntt_fwd_qr(c, ea, qr);
    orc_ntt_fwd_qr(c, ea + qrn, qr);
    orc_ntt_fwd_qr(c, eb, qr);
    orc_ntt_fwd_qr(c, eb + qrn, qr);
    if (a == b)
        tensor_limbs(s, qr, n, ea, ea, t3);
    else
        tensor_limbs(s, qr, n, ea, eb, t3);
    uint64_t *rt = malloc((size_t)nR * n * 8);
    uint64_t *o3 = malloc(3 * qn * 8);
    for (int p = 0; p < 3; p++) {
        orc_ntt_inv_qr(c, t3 + p * qrn, qr);
        orc_hps_scale_round_qr_r(c, t3 + p * qrn, rt);
        orc_hps_bconv_r_to_q(c, rt, o3 + p * qn);
    }
    orc_relinearize(c, nQ, o3, rlk, 1);
    memcpy(out, o3, 2 * qn * 8);
    free(ea); free(eb); free(t3); free(rt); free(o3);
}

/* ------------------------------------------------------------------ samplers and key generation */

/* The reference's generator (src/prng.cu:17-131): the Salsa20/20 core over a state whose words
 * 0-7 and 10-15 are the first 56 seed bytes (little-endian) and words 8-9 the 64-bit nonce, with
 * the input state added back; one call gives 16 output words. */
static uint32_t rotl32(uint32_t v, int c) { return (v << c) | (v >> (32 - c)); }

static void salsa_core(const uint8_t *seed, uint64_t nonce, uint32_t out[16]) {
    uint32_t s[16], x[16];
    for (int i = 0; i < 14; i++) {
        const uint8_t *b = seed + 4 * i;
        uint32_t w = (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
        s[i < 8 ? i : i + 2] = w;
    }
    s[8] = (uint32_t)nonce;
    s[9] = (uint32_t)(nonce >> 32);
    memcpy(x, s, sizeof(x));
    static const int qr[8][4] = {{0, 4, 8, 12}, {5, 9, 13, 1}, {10, 14, 2, 6}, {15, 3, 7, 11},
                                 {0, 1, 2, 3},  {5, 6, 7, 4},  {10, 11, 8, 9}, {15, 12, 13, 14}};
    for (int r = 0; r < 10; r++)
        for (int k = 0; k < 8; k++) {
            uint32_t *a = &x[qr[k][0]], *b = &x[qr[k][1]], *c = &x[qr[k][2]], *d = &x[qr[k][3]];
            *b ^= rotl32(*a + *d, 7);
            *c ^= rotl32(*b + *a, 9);
            *d ^= rotl32(*c + *b, 13);
            *a ^= rotl32(*d + *c, 18);
        }
    for (int i = 0; i < 16; i++) out[i] = x[i] + s[i];
}

void orc_sample_uniform(const orc_ctx *c, const uint8_t *seed, int limbs, uint64_t *out) {
    const size_t per = (size_t)c->n / 8, total = per * (size_t)limbs;
    const uint64_t retry = (uint64_t)limbs * (uint64_t)c->n;
    for (size_t t = 0; t < total; t++) {
        const uint64_t q = c->mod[t / per];
        const uint64_t limit = ~0ull - (~0ull % q) - 1;
        uint32_t w[16];
        salsa_core(seed, t, w);
        uint64_t tries = 1;
        for (int i = 0; i < 8; i++) {
            uint64_t v = (uint64_t)w[2 * i] | ((uint64_t)w[2 * i + 1] << 32);
            while (v > limit) { /* a whole new block, same word position (src/prng.cu:180-186) */
                salsa_core(seed, t + tries * retry, w);
                tries++;
                v = (uint64_t)w[2 * i] | ((uint64_t)w[2 * i + 1] << 32);
            }
            out[t * 8 + i] = v % q;
        }
    }
}

static int popc8(uint32_t b) { return __builtin_popcount(b & 0xFF); }

void orc_sample_small(const orc_ctx *c, const uint8_t *seed, int kind, int64_t *out) {
    for (int i = 0; i < c->n; i++) {
        uint32_t w[16];
        salsa_core(seed, (uint64_t)i, w);
        const uint32_t b0 = w[0] & 0xFF, b1 = (w[0] >> 8) & 0xFF, b2 = (w[0] >> 16) & 0xFF, b3 = w[0] >> 24;
        const uint32_t b4 = w[1] & 0xFF, b5 = (w[1] >> 8) & 0xFF;
        if (kind == 0)
            out[i] = (int64_t)(b0 % 3) - 1; /* src/prng.cu:146-153 */
        else
            out[i] = (int64_t)(popc8(b0) + popc8(b1) + popc8(b2 & 0x1F)) -
                     (int64_t)(popc8(b3) + popc8(b4) + popc8(b5 & 0x1F)); /* src/prng.cu:231-240 */
    }
}

/* generate_one_kswitch_key (src/secretkey.cu:297-341): key[d] = (-(a_d s + e_d) + (P mod q_j) s_src
 * on digit d's limbs, a_d); a [dnum][QP][N] NTT form, e_ntt [dnum][QP][N], s and s_src [QP][N]. */
void orc_kswitch_key_combine(const orc_ctx *c, const uint64_t *s, const uint64_t *s_src, const uint64_t *a,
                             const uint64_t *e_ntt, uint64_t *key) {
    const int qp = c->nQ + c->nP, dnum = (c->nQ + c->nP - 1) / c->nP;
    const size_t n = (size_t)c->n, qpn = (size_t)qp * n;
    for (int d = 0; d < dnum; d++)
        for (int j = 0; j < qp; j++) {
            const uint64_t q = c->mod[j];
            uint64_t pm = 1;
            for (int k = c->nQ; k < qp; k++) pm = orc_mulmod(pm, c->mod[k] % q, q);
            const int own = j < c->nQ && j >= d * c->nP && j < (d + 1) * c->nP;
            for (size_t i = 0; i < n; i++) {
                const size_t x = (size_t)j * n + i;
                const uint64_t as = (uint64_t)(((u128)a[d * qpn + x] * s[x] + e_ntt[d * qpn + x]) % q);
                uint64_t b = as ? q - as : 0;
                if (own) b = (uint64_t)(((u128)b + orc_mulmod(pm, s_src[x], q)) % q);
                key[2 * d * qpn + x] = b;
                key[2 * d * qpn + qpn + x] = a[d * qpn + x];
            }
        }
}
