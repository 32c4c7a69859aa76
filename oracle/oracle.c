/*
 * CPU oracle for the BLS12-381 prover hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's CPU semantics, used by tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline leg to check results.
 * Nothing in the product links it.  Each function names the reference
 * file:line it follows (paths relative to the dcSpark/midnight-ledger-cuda
 * tree).  The reference CPU arithmetic lives in blst 0.3.16 (a Cargo.lock
 * dependency that is not vendored); its published algorithms -- Montgomery
 * multiplication over 64-bit limbs, Jacobian point formulas, zcash point
 * encodings -- are restated here from their public definitions.
 */
#include "oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

typedef unsigned __int128 u128;
typedef uint64_t u64;

/* ======================================================================== */
/* Generic Montgomery arithmetic over n <= 6 64-bit limbs                    */
/* ======================================================================== */

typedef struct {
    int n;
    u64 p[6];
    u64 inv;    /* -p^-1 mod 2^64 */
    u64 one[6]; /* R mod p */
    u64 r2[6];  /* R^2 mod p */
} field_t;

static field_t FR, FP;
static pthread_once_t init_once = PTHREAD_ONCE_INIT;

static int mp_geq(const u64 *a, const u64 *b, int n)
{
    for (int i = n - 1; i >= 0; i--) {
        if (a[i] != b[i]) return a[i] > b[i];
    }
    return 1;
}

static u64 mp_add(u64 *out, const u64 *a, const u64 *b, int n)
{
    u64 c = 0;
    for (int i = 0; i < n; i++) {
        u128 v = (u128)a[i] + b[i] + c;
        out[i] = (u64)v;
        c = (u64)(v >> 64);
    }
    return c;
}

static u64 mp_sub(u64 *out, const u64 *a, const u64 *b, int n)
{
    u64 br = 0;
    for (int i = 0; i < n; i++) {
        u128 v = (u128)a[i] - b[i] - br;
        out[i] = (u64)v;
        br = (u64)(v >> 64) & 1;
    }
    return br;
}

static int mp_is_zero(const u64 *a, int n)
{
    u64 x = 0;
    for (int i = 0; i < n; i++) x |= a[i];
    return x == 0;
}

static void f_add(u64 *out, const u64 *a, const u64 *b, const field_t *F)
{
    u64 t[6];
    u64 c = mp_add(t, a, b, F->n);
    if (c || mp_geq(t, F->p, F->n)) mp_sub(t, t, F->p, F->n);
    memcpy(out, t, 8 * F->n);
}

static void f_sub(u64 *out, const u64 *a, const u64 *b, const field_t *F)
{
    u64 t[6];
    if (mp_sub(t, a, b, F->n)) mp_add(t, t, F->p, F->n);
    memcpy(out, t, 8 * F->n);
}

static void f_neg(u64 *out, const u64 *a, const field_t *F)
{
    if (mp_is_zero(a, F->n)) { memset(out, 0, 8 * F->n); return; }
    mp_sub(out, F->p, a, F->n);
}

/* CIOS Montgomery multiplication: out = a*b*R^-1 mod p, fully reduced. */
/* CIOS Montgomery product for a limb count n known where it is inlined, so
 * that the loops unroll (the generic entry below dispatches on F->n) */
static inline __attribute__((always_inline)) void f_mul_n(u64 *out, const u64 *a, const u64 *b,
                                                          const field_t *F, const int n)
{
    u64 t[8] = {0};
    for (int i = 0; i < n; i++) {
        u64 carry = 0;
        for (int j = 0; j < n; j++) {
            u128 v = (u128)a[j] * b[i] + t[j] + carry;
            t[j] = (u64)v;
            carry = (u64)(v >> 64);
        }
        u128 v = (u128)t[n] + carry;
        t[n] = (u64)v;
        t[n + 1] = (u64)(v >> 64);
        u64 m = t[0] * F->inv;
        v = (u128)m * F->p[0] + t[0];
        carry = (u64)(v >> 64);
        for (int j = 1; j < n; j++) {
            v = (u128)m * F->p[j] + t[j] + carry;
            t[j - 1] = (u64)v;
            carry = (u64)(v >> 64);
        }
        v = (u128)t[n] + carry;
        t[n - 1] = (u64)v;
        t[n] = t[n + 1] + (u64)(v >> 64);
    }
    if (t[n] || mp_geq(t, F->p, n)) mp_sub(t, t, F->p, n);
    memcpy(out, t, 8 * n);
}

static void f_mul(u64 *out, const u64 *a, const u64 *b, const field_t *F)
{
    if (F->n == 6) f_mul_n(out, a, b, F, 6);
    else if (F->n == 4) f_mul_n(out, a, b, F, 4);
    else f_mul_n(out, a, b, F, F->n);
}

/* exponent given as little-endian u64 limbs */
static void f_pow(u64 *out, const u64 *a, const u64 *exp, int elimbs, const field_t *F)
{
    u64 acc[6], base[6];
    memcpy(acc, F->one, 8 * F->n);
    memcpy(base, a, 8 * F->n);
    for (int i = elimbs * 64 - 1; i >= 0; i--) {
        f_mul(acc, acc, acc, F);
        if ((exp[i / 64] >> (i % 64)) & 1) f_mul(acc, acc, base, F);
    }
    memcpy(out, acc, 8 * F->n);
}

/* Fermat inversion a^(p-2); 0 maps to 0 (as blst's inverse does). */
static void f_inv(u64 *out, const u64 *a, const field_t *F)
{
    u64 e[6];
    u64 two[6] = {2, 0, 0, 0, 0, 0};
    mp_sub(e, F->p, two, F->n);
    f_pow(out, a, e, F->n, F);
}

static void f_to_mont(u64 *out, const u64 *a, const field_t *F) { f_mul(out, a, F->r2, F); }

static void f_from_mont(u64 *out, const u64 *a, const field_t *F)
{
    u64 one[6] = {1, 0, 0, 0, 0, 0};
    f_mul(out, a, one, F);
}

static void parse_hex(u64 *out, int n, const char *hex)
{
    memset(out, 0, 8 * n);
    size_t len = strlen(hex);
    for (size_t k = 0; k < len; k++) {
        char ch = hex[len - 1 - k];
        u64 v = (ch >= '0' && ch <= '9') ? (u64)(ch - '0')
              : (ch >= 'a' && ch <= 'f') ? (u64)(ch - 'a' + 10)
              : (u64)(ch - 'A' + 10);
        out[k / 16] |= v << (4 * (k % 16));
    }
}

static void field_init(field_t *F, int n, const char *modulus_hex)
{
    F->n = n;
    parse_hex(F->p, n, modulus_hex);
    /* -p^-1 mod 2^64 by Newton iteration */
    u64 x = 1;
    for (int i = 0; i < 7; i++) x *= 2 - F->p[0] * x;
    F->inv = (u64)0 - x;
    /* R mod p = 2^(64n) mod p by doubling 1, R^2 by doubling further */
    u64 t[6] = {1, 0, 0, 0, 0, 0};
    for (int i = 0; i < 64 * n; i++) f_add(t, t, t, F);
    memcpy(F->one, t, 8 * n);
    for (int i = 0; i < 64 * n; i++) f_add(t, t, t, F);
    memcpy(F->r2, t, 8 * n);
}

/* Curve constants (public BLS12-381 parameters). */
static const char *FR_MODULUS = "73eda753299d7d483339d80809a1d80553bda402fffe5bfeffffffff00000001";
static const char *FP_MODULUS =
    "1a0111ea397fe69a4b1ba7b6434bacd764774b84f38512bf6730d2a0f6b0f6241eabfffeb153ffffb9feffffffffaaab";
static const char *G1_X =
    "17f1d3a73197d7942695638c4fa9ac0fc3688c4f9774b905a14e3a3f171bac586c55e83ff97a1aeffb3af00adb22c6bb";
static const char *G1_Y =
    "08b3f481e3aaa0f1a09e30ed741d8ae4fcf5e095d5d00af600db18cb2c04b3edd03cc744a2888ae40caa232946c5e7e1";

static u64 FP_B[6];        /* 4 in Montgomery form */
static orc_g1_affine G1_GEN;
static orc_fr FR_CONST[7];

static void oracle_init(void)
{
    field_init(&FR, 4, FR_MODULUS);
    field_init(&FP, 6, FP_MODULUS);
    u64 four[6] = {4, 0, 0, 0, 0, 0};
    f_to_mont(FP_B, four, &FP);
    u64 t[6];
    parse_hex(t, 6, G1_X);
    f_to_mont(G1_GEN.x.l, t, &FP);
    parse_hex(t, 6, G1_Y);
    f_to_mont(G1_GEN.y.l, t, &FP);

    /* Fr constants (fq.rs:31-33,70,481-501,693-702): generator 7, the 2^32-th
     * root of unity 7^t (r - 1 = t * 2^32), its inverse, DELTA = 7^(2^32),
     * ZETA = 7^((r-1)/3) and 1/2.  Their Montgomery limbs are pinned against
     * the reference's literal constants by tests/test_oracle.py. */
    u64 c[4];
    memcpy(FR_CONST[0].l, FR.one, 32);
    u64 seven[4] = {7, 0, 0, 0};
    f_to_mont(FR_CONST[1].l, seven, &FR);
    u64 rm1[4], one_c[4] = {1, 0, 0, 0};
    mp_sub(rm1, FR.p, one_c, 4);
    /* t = (r-1) >> 32 */
    u64 texp[4];
    for (int i = 0; i < 4; i++) {
        texp[i] = (rm1[i] >> 32) | (i + 1 < 4 ? rm1[i + 1] << 32 : 0);
    }
    f_pow(FR_CONST[2].l, FR_CONST[1].l, texp, 4, &FR);
    f_inv(FR_CONST[3].l, FR_CONST[2].l, &FR);
    u64 e32[4] = {(u64)1 << 32, 0, 0, 0};
    f_pow(FR_CONST[4].l, FR_CONST[1].l, e32, 4, &FR);
    /* (r-1)/3 */
    {
        u128 rem = 0;
        for (int i = 3; i >= 0; i--) {
            u128 cur = (rem << 64) | rm1[i];
            c[i] = (u64)(cur / 3);
            rem = cur % 3;
        }
    }
    f_pow(FR_CONST[5].l, FR_CONST[1].l, c, 4, &FR);
    u64 two[4] = {2, 0, 0, 0}, two_m[4];
    f_to_mont(two_m, two, &FR);
    f_inv(FR_CONST[6].l, two_m, &FR);
}

#define INIT() pthread_once(&init_once, oracle_init)

/* ======================================================================== */
/* Fr / Fp exported wrappers                                                 */
/* ======================================================================== */

void orc_fr_mul(orc_fr *o, const orc_fr *a, const orc_fr *b) { INIT(); f_mul(o->l, a->l, b->l, &FR); }
void orc_fr_add(orc_fr *o, const orc_fr *a, const orc_fr *b) { INIT(); f_add(o->l, a->l, b->l, &FR); }
void orc_fr_sub(orc_fr *o, const orc_fr *a, const orc_fr *b) { INIT(); f_sub(o->l, a->l, b->l, &FR); }
void orc_fr_inv(orc_fr *o, const orc_fr *a) { INIT(); f_inv(o->l, a->l, &FR); }
void orc_fr_to_mont(orc_fr *o, const orc_fr *a) { INIT(); f_to_mont(o->l, a->l, &FR); }
void orc_fr_from_mont(orc_fr *o, const orc_fr *a) { INIT(); f_from_mont(o->l, a->l, &FR); }
void orc_fr_from_u64(orc_fr *o, uint64_t v)
{
    INIT();
    u64 t[4] = {v, 0, 0, 0};
    f_to_mont(o->l, t, &FR);
}
void orc_fr_pow(orc_fr *o, const orc_fr *a, const uint64_t *e, size_t el)
{
    INIT();
    f_pow(o->l, a->l, e, (int)el, &FR);
}
int orc_fr_constant(orc_fr *o, int which)
{
    INIT();
    if (which < 0 || which > 6) return -1;
    *o = FR_CONST[which];
    return 0;
}

void orc_fr_from_uniform_bytes(orc_fr *out, const uint8_t bytes[64])
{
    /* fq.rs:704-725: a0, a1 are the raw little-endian limbs of each half,
     * interpreted as Montgomery values; result = a0*R2 + a1*R3 (Montgomery). */
    INIT();
    u64 a0[4], a1[4], r3[4], t0[4], t1[4];
    for (int i = 0; i < 4; i++) {
        a0[i] = 0;
        a1[i] = 0;
        for (int b = 0; b < 8; b++) {
            a0[i] |= (u64)bytes[8 * i + b] << (8 * b);
            a1[i] |= (u64)bytes[32 + 8 * i + b] << (8 * b);
        }
    }
    /* R3 = R^3 mod r in Montgomery form means value R^3 * R... fq.rs stores
     * R3 as the limbs of 2^768 mod r; mul(x, R3) = x * 2^768 * 2^-256. */
    u64 one[4] = {1, 0, 0, 0};
    /* 2^768 mod r: double FR.r2 (2^512) 256 times */
    memcpy(r3, FR.r2, 32);
    for (int i = 0; i < 256; i++) f_add(r3, r3, r3, &FR);
    (void)one;
    f_mul(t0, a0, FR.r2, &FR);
    f_mul(t1, a1, r3, &FR);
    f_add(out->l, t0, t1, &FR);
}

int orc_fr_cmp_canonical(const orc_fr *a, const orc_fr *b)
{
    /* fq.rs:152-164 compares the big-endian canonical byte strings */
    INIT();
    u64 x[4], y[4];
    f_from_mont(x, a->l, &FR);
    f_from_mont(y, b->l, &FR);
    for (int i = 3; i >= 0; i--) {
        if (x[i] != y[i]) return x[i] < y[i] ? -1 : 1;
    }
    return 0;
}

void orc_fp_mul(orc_fp *o, const orc_fp *a, const orc_fp *b) { INIT(); f_mul(o->l, a->l, b->l, &FP); }
void orc_fp_to_mont(orc_fp *o, const orc_fp *a) { INIT(); f_to_mont(o->l, a->l, &FP); }
void orc_fp_from_mont(orc_fp *o, const orc_fp *a) { INIT(); f_from_mont(o->l, a->l, &FP); }

int orc_fp_sqrt(orc_fp *out, const orc_fp *a)
{
    /* p = 3 mod 4, so sqrt(a) = a^((p+1)/4) when a is a square. */
    INIT();
    u64 e[6], one[6] = {1, 0, 0, 0, 0, 0}, s[6], chk[6];
    mp_add(e, FP.p, one, 6);
    for (int i = 0; i < 6; i++) e[i] = (e[i] >> 2) | (i + 1 < 6 ? e[i + 1] << 62 : 0);
    f_pow(s, a->l, e, 6, &FP);
    f_mul(chk, s, s, &FP);
    memcpy(out->l, s, 48);
    return memcmp(chk, a->l, 48) == 0;
}

/* ======================================================================== */
/* G1 (y^2 = x^3 + 4) in Jacobian coordinates                                */
/* ======================================================================== */

static const u64 ZERO6[6] = {0};

void orc_g1_generator(orc_g1_affine *out)
{
    INIT();
    *out = G1_GEN;
}

static int aff_is_inf(const orc_g1_affine *p)
{
    return mp_is_zero(p->x.l, 6) && mp_is_zero(p->y.l, 6);
}

int orc_g1_is_on_curve(const orc_g1_affine *p)
{
    INIT();
    if (aff_is_inf(p)) return 1;
    u64 y2[6], x3[6];
    f_mul(y2, p->y.l, p->y.l, &FP);
    f_mul(x3, p->x.l, p->x.l, &FP);
    f_mul(x3, x3, p->x.l, &FP);
    f_add(x3, x3, FP_B, &FP);
    return memcmp(x3, y2, 48) == 0;
}

static void jac_set_inf(orc_g1_jac *p)
{
    memset(p, 0, sizeof(*p));
    memcpy(p->x.l, FP.one, 48);
    memcpy(p->y.l, FP.one, 48);
}

static int jac_is_inf(const orc_g1_jac *p) { return mp_is_zero(p->z.l, 6); }

void orc_g1_from_affine(orc_g1_jac *out, const orc_g1_affine *p)
{
    INIT();
    if (aff_is_inf(p)) { jac_set_inf(out); return; }
    out->x = p->x;
    out->y = p->y;
    memcpy(out->z.l, FP.one, 48);
}

/* dbl-2009-l (a = 0): 2M + 5S */
static void jac_double(orc_g1_jac *r, const orc_g1_jac *p)
{
    if (jac_is_inf(p)) { *r = *p; return; }
    u64 A[6], B[6], C[6], D[6], E[6], F_[6], t[6], X3[6], Y3[6], Z3[6];
    f_mul(A, p->x.l, p->x.l, &FP);
    f_mul(B, p->y.l, p->y.l, &FP);
    f_mul(C, B, B, &FP);
    f_add(t, p->x.l, B, &FP);
    f_mul(t, t, t, &FP);
    f_sub(t, t, A, &FP);
    f_sub(t, t, C, &FP);
    f_add(D, t, t, &FP);
    f_add(E, A, A, &FP);
    f_add(E, E, A, &FP);
    f_mul(F_, E, E, &FP);
    f_add(t, D, D, &FP);
    f_sub(X3, F_, t, &FP);
    f_sub(t, D, X3, &FP);
    f_mul(t, E, t, &FP);
    u64 c8[6];
    f_add(c8, C, C, &FP);
    f_add(c8, c8, c8, &FP);
    f_add(c8, c8, c8, &FP);
    f_sub(Y3, t, c8, &FP);
    f_mul(Z3, p->y.l, p->z.l, &FP);
    f_add(Z3, Z3, Z3, &FP);
    memcpy(r->x.l, X3, 48);
    memcpy(r->y.l, Y3, 48);
    memcpy(r->z.l, Z3, 48);
}

/* add-2007-bl general addition, with the doubling and inverse cases handled */
static void jac_add(orc_g1_jac *r, const orc_g1_jac *p, const orc_g1_jac *q)
{
    if (jac_is_inf(p)) { *r = *q; return; }
    if (jac_is_inf(q)) { *r = *p; return; }
    u64 Z1Z1[6], Z2Z2[6], U1[6], U2[6], S1[6], S2[6], H[6], I[6], J[6], rr[6], V[6], t[6];
    f_mul(Z1Z1, p->z.l, p->z.l, &FP);
    f_mul(Z2Z2, q->z.l, q->z.l, &FP);
    f_mul(U1, p->x.l, Z2Z2, &FP);
    f_mul(U2, q->x.l, Z1Z1, &FP);
    f_mul(S1, p->y.l, q->z.l, &FP);
    f_mul(S1, S1, Z2Z2, &FP);
    f_mul(S2, q->y.l, p->z.l, &FP);
    f_mul(S2, S2, Z1Z1, &FP);
    f_sub(H, U2, U1, &FP);
    f_sub(rr, S2, S1, &FP);
    if (mp_is_zero(H, 6)) {
        if (mp_is_zero(rr, 6)) { jac_double(r, p); return; }
        jac_set_inf(r);
        return;
    }
    f_add(I, H, H, &FP);
    f_mul(I, I, I, &FP);
    f_mul(J, H, I, &FP);
    f_add(rr, rr, rr, &FP);
    f_mul(V, U1, I, &FP);
    u64 X3[6], Y3[6], Z3[6];
    f_mul(X3, rr, rr, &FP);
    f_sub(X3, X3, J, &FP);
    f_sub(X3, X3, V, &FP);
    f_sub(X3, X3, V, &FP);
    f_sub(t, V, X3, &FP);
    f_mul(Y3, rr, t, &FP);
    f_mul(t, S1, J, &FP);
    f_add(t, t, t, &FP);
    f_sub(Y3, Y3, t, &FP);
    f_add(Z3, p->z.l, q->z.l, &FP);
    f_mul(Z3, Z3, Z3, &FP);
    f_sub(Z3, Z3, Z1Z1, &FP);
    f_sub(Z3, Z3, Z2Z2, &FP);
    f_mul(Z3, Z3, H, &FP);
    memcpy(r->x.l, X3, 48);
    memcpy(r->y.l, Y3, 48);
    memcpy(r->z.l, Z3, 48);
}

static void jac_add_aff(orc_g1_jac *r, const orc_g1_jac *p, const orc_g1_affine *q)
{
    if (aff_is_inf(q)) { *r = *p; return; }
    orc_g1_jac qj;
    qj.x = q->x;
    qj.y = q->y;
    memcpy(qj.z.l, FP.one, 48);
    jac_add(r, p, &qj);
}

static void jac_neg(orc_g1_jac *r, const orc_g1_jac *p)
{
    *r = *p;
    f_neg(r->y.l, p->y.l, &FP);
}

void orc_g1_add(orc_g1_jac *o, const orc_g1_jac *a, const orc_g1_jac *b) { INIT(); jac_add(o, a, b); }
void orc_g1_add_affine(orc_g1_jac *o, const orc_g1_jac *a, const orc_g1_affine *b) { INIT(); jac_add_aff(o, a, b); }
void orc_g1_double(orc_g1_jac *o, const orc_g1_jac *a) { INIT(); jac_double(o, a); }
void orc_g1_neg(orc_g1_jac *o, const orc_g1_jac *a) { INIT(); jac_neg(o, a); }

void orc_g1_to_affine(orc_g1_affine *out, const orc_g1_jac *p)
{
    INIT();
    if (jac_is_inf(p)) { memset(out, 0, sizeof(*out)); return; }
    u64 zi[6], zi2[6], zi3[6];
    f_inv(zi, p->z.l, &FP);
    f_mul(zi2, zi, zi, &FP);
    f_mul(zi3, zi2, zi, &FP);
    f_mul(out->x.l, p->x.l, zi2, &FP);
    f_mul(out->y.l, p->y.l, zi3, &FP);
}

void orc_g1_jac_to_affine_batch(orc_g1_affine *out, const orc_g1_jac *p, size_t n)
{
    INIT();
    if (n == 0) return;
    /* Montgomery batch inversion of the z coordinates (skipping infinities) */
    u64 *pref = (u64 *)malloc(sizeof(u64) * 6 * n);
    u64 acc[6];
    memcpy(acc, FP.one, 48);
    for (size_t i = 0; i < n; i++) {
        memcpy(pref + 6 * i, acc, 48);
        if (!jac_is_inf(&p[i])) f_mul(acc, acc, p[i].z.l, &FP);
    }
    u64 inv[6];
    f_inv(inv, acc, &FP);
    for (size_t k = n; k-- > 0;) {
        if (jac_is_inf(&p[k])) { memset(&out[k], 0, sizeof(out[k])); continue; }
        u64 zi[6], zi2[6], zi3[6];
        f_mul(zi, inv, pref + 6 * k, &FP);
        f_mul(inv, inv, p[k].z.l, &FP);
        f_mul(zi2, zi, zi, &FP);
        f_mul(zi3, zi2, zi, &FP);
        f_mul(out[k].x.l, p[k].x.l, zi2, &FP);
        f_mul(out[k].y.l, p[k].y.l, zi3, &FP);
    }
    free(pref);
}

int orc_g1_affine_eq(const orc_g1_affine *a, const orc_g1_affine *b)
{
    return memcmp(a, b, sizeof(*a)) == 0;
}

int orc_g1_jac_eq(const orc_g1_jac *a, const orc_g1_jac *b)
{
    orc_g1_affine x, y;
    orc_g1_to_affine(&x, a);
    orc_g1_to_affine(&y, b);
    return orc_g1_affine_eq(&x, &y);
}

void orc_g1_mul(orc_g1_jac *out, const orc_g1_affine *p, const orc_fr *scalar)
{
    INIT();
    u64 s[4];
    f_from_mont(s, scalar->l, &FR);
    orc_g1_jac acc;
    jac_set_inf(&acc);
    for (int i = 255; i >= 0; i--) {
        jac_double(&acc, &acc);
        if ((s[i / 64] >> (i % 64)) & 1) jac_add_aff(&acc, &acc, p);
    }
    *out = acc;
}

/* ---- simple parallel-for ---- */
typedef struct {
    void (*fn)(void *ctx, size_t begin, size_t end);
    void *ctx;
    size_t begin, end;
} par_task;

static void *par_thread(void *arg)
{
    par_task *t = (par_task *)arg;
    t->fn(t->ctx, t->begin, t->end);
    return NULL;
}

static void parallel_for(size_t n, int threads, void (*fn)(void *, size_t, size_t), void *ctx)
{
    if (threads < 1) threads = 1;
    if ((size_t)threads > n) threads = (int)(n ? n : 1);
    if (threads == 1) { fn(ctx, 0, n); return; }
    pthread_t *tid = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    par_task *task = (par_task *)malloc(sizeof(par_task) * threads);
    for (int t = 0; t < threads; t++) {
        task[t].fn = fn;
        task[t].ctx = ctx;
        task[t].begin = n * t / threads;
        task[t].end = n * (t + 1) / threads;
        pthread_create(&tid[t], NULL, par_thread, &task[t]);
    }
    for (int t = 0; t < threads; t++) pthread_join(tid[t], NULL);
    free(tid);
    free(task);
}

/* fixed-base table for [s]G: TABLE[w][d] = d * 2^(8w) * G, d in 0..255 */
static orc_g1_affine *GEN_TABLE;
static pthread_once_t gen_table_once = PTHREAD_ONCE_INIT;

static void gen_table_init(void)
{
    orc_g1_jac *jt = (orc_g1_jac *)malloc(sizeof(orc_g1_jac) * 32 * 256);
    orc_g1_jac base;
    orc_g1_from_affine(&base, &G1_GEN);
    for (int w = 0; w < 32; w++) {
        jac_set_inf(&jt[w * 256]);
        for (int d = 1; d < 256; d++) jac_add(&jt[w * 256 + d], &jt[w * 256 + d - 1], &base);
        for (int k = 0; k < 8; k++) jac_double(&base, &base);
    }
    GEN_TABLE = (orc_g1_affine *)malloc(sizeof(orc_g1_affine) * 32 * 256);
    orc_g1_jac_to_affine_batch(GEN_TABLE, jt, 32 * 256);
    free(jt);
}

typedef struct {
    orc_g1_affine *out;
    const orc_fr *scalars;
} genmul_ctx;

static void genmul_range(void *vctx, size_t b, size_t e)
{
    genmul_ctx *c = (genmul_ctx *)vctx;
    size_t n = e - b;
    if (!n) return;
    orc_g1_jac *tmp = (orc_g1_jac *)malloc(sizeof(orc_g1_jac) * n);
    for (size_t i = b; i < e; i++) {
        u64 s[4];
        f_from_mont(s, c->scalars[i].l, &FR);
        orc_g1_jac acc;
        jac_set_inf(&acc);
        for (int w = 0; w < 32; w++) {
            unsigned d = (unsigned)((s[w / 8] >> (8 * (w % 8))) & 0xff);
            if (d) jac_add_aff(&acc, &acc, &GEN_TABLE[w * 256 + d]);
        }
        tmp[i - b] = acc;
    }
    orc_g1_jac_to_affine_batch(c->out + b, tmp, n);
    free(tmp);
}

void orc_g1_generator_mul_batch(orc_g1_affine *out, const orc_fr *scalars, size_t n, int threads)
{
    INIT();
    pthread_once(&gen_table_once, gen_table_init);
    genmul_ctx c = {out, scalars};
    parallel_for(n, threads, genmul_range, &c);
}

/* ---- zcash serialisation (g1.rs:1179-1211; blst p1 (de)serialisation) ---- */

static void fp_to_be(uint8_t out[48], const u64 *mont)
{
    u64 c[6];
    f_from_mont(c, mont, &FP);
    for (int i = 0; i < 48; i++) out[47 - i] = (uint8_t)(c[i / 8] >> (8 * (i % 8)));
}

static int fp_from_be(u64 *mont, const uint8_t in[48])
{
    u64 c[6] = {0};
    for (int i = 0; i < 48; i++) c[i / 8] |= (u64)in[47 - i] << (8 * (i % 8));
    if (mp_geq(c, FP.p, 6)) return 1;
    f_to_mont(mont, c, &FP);
    return 0;
}

/* y is "lexicographically largest" when y > (p-1)/2, i.e. y > p - y */
static int fp_lexicographically_largest(const u64 *mont)
{
    u64 c[6], neg[6];
    f_from_mont(c, mont, &FP);
    if (mp_is_zero(c, 6)) return 0;
    mp_sub(neg, FP.p, c, 6);
    return !mp_geq(neg, c, 6);
}

int orc_g1_decompress(orc_g1_affine *out, const uint8_t in[48])
{
    INIT();
    uint8_t buf[48];
    memcpy(buf, in, 48);
    int compressed = (buf[0] >> 7) & 1, infinity = (buf[0] >> 6) & 1, sort = (buf[0] >> 5) & 1;
    if (!compressed) return 1;
    buf[0] &= 0x1f;
    if (infinity) {
        for (int i = 0; i < 48; i++) if (buf[i]) return 2;
        if (sort) return 2;
        memset(out, 0, sizeof(*out));
        return 0;
    }
    u64 x[6], rhs[6], y[6];
    if (fp_from_be(x, buf)) return 3;
    f_mul(rhs, x, x, &FP);
    f_mul(rhs, rhs, x, &FP);
    f_add(rhs, rhs, FP_B, &FP);
    orc_fp r, s;
    memcpy(r.l, rhs, 48);
    if (!orc_fp_sqrt(&s, &r)) return 4;
    memcpy(y, s.l, 48);
    if (fp_lexicographically_largest(y) != sort) f_neg(y, y, &FP);
    memcpy(out->x.l, x, 48);
    memcpy(out->y.l, y, 48);
    return 0;
}

void orc_g1_compress(uint8_t out[48], const orc_g1_affine *p)
{
    INIT();
    if (aff_is_inf(p)) {
        memset(out, 0, 48);
        out[0] = 0xc0;
        return;
    }
    fp_to_be(out, p->x.l);
    out[0] |= 0x80;
    if (fp_lexicographically_largest(p->y.l)) out[0] |= 0x20;
}

int orc_g1_from_uncompressed(orc_g1_affine *out, const uint8_t in[96])
{
    INIT();
    uint8_t buf[96];
    memcpy(buf, in, 96);
    if ((buf[0] >> 7) & 1) return 1;
    int infinity = (buf[0] >> 6) & 1;
    if ((buf[0] >> 5) & 1) return 2;
    buf[0] &= 0x1f;
    if (infinity) {
        for (int i = 0; i < 96; i++) if (buf[i]) return 2;
        memset(out, 0, sizeof(*out));
        return 0;
    }
    if (fp_from_be(out->x.l, buf) || fp_from_be(out->y.l, buf + 48)) return 3;
    if (!orc_g1_is_on_curve(out)) return 4;
    return 0;
}

void orc_g1_to_uncompressed(uint8_t out[96], const orc_g1_affine *p)
{
    INIT();
    if (aff_is_inf(p)) {
        memset(out, 0, 96);
        out[0] = 0x40;
        return;
    }
    fp_to_be(out, p->x.l);
    fp_to_be(out + 48, p->y.l);
}

/* ======================================================================== */
/* Multiexp                                                                  */
/* ======================================================================== */

int32_t orc_booth_index(size_t window_index, size_t window_size, const uint8_t el[32])
{
    /* msm.rs:13-56: a (window_size + 1)-bit slice overlapping the previous
     * window by one bit, with an implicit zero below bit 0. */
    size_t skip_bits = window_index * window_size;
    skip_bits = skip_bits ? skip_bits - 1 : 0;
    size_t skip_bytes = skip_bits / 8;
    uint8_t v[4] = {0, 0, 0, 0};
    for (size_t i = 0; i < 4 && skip_bytes + i < 32; i++) v[i] = el[skip_bytes + i];
    uint32_t tmp = (uint32_t)v[0] | ((uint32_t)v[1] << 8) | ((uint32_t)v[2] << 16) | ((uint32_t)v[3] << 24);
    if (window_index == 0) tmp <<= 1;
    tmp >>= skip_bits - skip_bytes * 8;
    tmp &= (1u << (window_size + 1)) - 1;
    int positive = (tmp & (1u << window_size)) == 0;
    tmp = (tmp + 1) >> 1;
    if (positive) return (int32_t)tmp;
    return -(int32_t)((~(tmp - 1)) & ((1u << window_size) - 1));
}

void orc_g1_msm_naive(orc_g1_jac *out, const orc_g1_affine *bases, const orc_fr *scalars, size_t n)
{
    INIT();
    orc_g1_jac acc, t;
    jac_set_inf(&acc);
    for (size_t i = 0; i < n; i++) {
        orc_g1_mul(&t, &bases[i], &scalars[i]);
        jac_add(&acc, &acc, &t);
    }
    *out = acc;
}

typedef struct {
    const orc_g1_affine *bases;
    const uint8_t *bytes; /* canonical LE scalars, 32 bytes each */
    size_t n;
    int c;
    int nwin;
    int chunks;
    orc_g1_jac *partial; /* [nwin * chunks] */
} msm_ctx;

static void msm_task_range(void *vctx, size_t b, size_t e)
{
    msm_ctx *m = (msm_ctx *)vctx;
    size_t nb = (size_t)1 << (m->c - 1);
    orc_g1_jac *buckets = (orc_g1_jac *)malloc(sizeof(orc_g1_jac) * nb);
    for (size_t task = b; task < e; task++) {
        int w = (int)(task / m->chunks);
        int ch = (int)(task % m->chunks);
        size_t lo = m->n * ch / m->chunks, hi = m->n * (ch + 1) / m->chunks;
        for (size_t k = 0; k < nb; k++) jac_set_inf(&buckets[k]);
        for (size_t i = lo; i < hi; i++) {
            int32_t idx = orc_booth_index((size_t)w, (size_t)m->c, m->bytes + 32 * i);
            if (idx == 0) continue;
            orc_g1_affine p = m->bases[i];
            if (idx < 0) {
                if (!aff_is_inf(&p)) f_neg(p.y.l, p.y.l, &FP);
                idx = -idx;
            }
            jac_add_aff(&buckets[idx - 1], &buckets[idx - 1], &p);
        }
        /* summation by parts (msm.rs:528-536) */
        orc_g1_jac run, acc;
        jac_set_inf(&run);
        jac_set_inf(&acc);
        for (size_t k = nb; k-- > 0;) {
            jac_add(&run, &run, &buckets[k]);
            jac_add(&acc, &acc, &run);
        }
        m->partial[task] = acc;
    }
    free(buckets);
}

void orc_g1_msm(orc_g1_jac *out, const orc_g1_affine *bases, const orc_fr *scalars, size_t n,
                int threads, int window_bits)
{
    INIT();
    if (n == 0) { jac_set_inf(out); return; }
    int c = window_bits;
    if (c <= 0) {
        /* msm.rs:489-495 window choice */
        c = n < 4 ? 1 : n < 32 ? 3 : (int)ceil(log((double)n));
    }
    if (c > 20) c = 20;
    uint8_t *bytes = (uint8_t *)malloc(32 * n);
    for (size_t i = 0; i < n; i++) {
        u64 s[4];
        f_from_mont(s, scalars[i].l, &FR);
        for (int k = 0; k < 32; k++) bytes[32 * i + k] = (uint8_t)(s[k / 8] >> (8 * (k % 8)));
    }
    msm_ctx m;
    m.bases = bases;
    m.bytes = bytes;
    m.n = n;
    m.c = c;
    m.nwin = 255 / c + 1; /* NUM_BITS / c + 1 (msm.rs:505) */
    if (threads < 1) threads = 1;
    m.chunks = (2 * threads + m.nwin - 1) / m.nwin;
    if ((size_t)m.chunks > n) m.chunks = (int)n;
    if (m.chunks < 1) m.chunks = 1;
    size_t tasks = (size_t)m.nwin * m.chunks;
    m.partial = (orc_g1_jac *)malloc(sizeof(orc_g1_jac) * tasks);
    parallel_for(tasks, threads, msm_task_range, &m);
    orc_g1_jac acc;
    jac_set_inf(&acc);
    for (int w = m.nwin - 1; w >= 0; w--) {
        for (int k = 0; k < c; k++) jac_double(&acc, &acc);
        for (int ch = 0; ch < m.chunks; ch++) jac_add(&acc, &acc, &m.partial[w * m.chunks + ch]);
    }
    *out = acc;
    free(m.partial);
    free(bytes);
}

/* ======================================================================== */
/* FFT / evaluation domain                                                   */
/* ======================================================================== */

static size_t bitrev(size_t x, unsigned bits)
{
    size_t r = 0;
    for (unsigned i = 0; i < bits; i++) {
        r = (r << 1) | (x & 1);
        x >>= 1;
    }
    return r;
}

typedef struct {
    orc_fr *a;
    const orc_fr *tw;
    size_t n;
    unsigned log_n;
    unsigned stage;
} fft_ctx;

static void fft_stage_range(void *vctx, size_t b, size_t e)
{
    /* butterfly index t in [0, n/2): group g, offset j within a half of size m */
    fft_ctx *c = (fft_ctx *)vctx;
    size_t m = (size_t)1 << c->stage; /* half size */
    size_t step = c->n / (2 * m);     /* twiddle stride */
    for (size_t t = b; t < e; t++) {
        size_t g = t / m, j = t % m;
        size_t i0 = g * 2 * m + j, i1 = i0 + m;
        u64 x[4];
        f_mul(x, c->a[i1].l, c->tw[j * step].l, &FR);
        f_sub(c->a[i1].l, c->a[i0].l, x, &FR);
        f_add(c->a[i0].l, c->a[i0].l, x, &FR);
    }
}

typedef struct {
    orc_fr *tw;
    const orc_fr *omega;
    size_t half;
    int threads;
} tw_ctx;

static void tw_range(void *vctx, size_t b, size_t e)
{
    tw_ctx *c = (tw_ctx *)vctx;
    u64 w[4];
    u64 eb[1] = {b};
    f_pow(w, c->omega->l, eb, 1, &FR);
    for (size_t j = b; j < e; j++) {
        memcpy(c->tw[j].l, w, 32);
        f_mul(w, w, c->omega->l, &FR);
    }
}

void orc_fr_fft(orc_fr *a, uint32_t log_n, const orc_fr *omega, int threads)
{
    /* fft.rs:35-113 (best_fft): bit-reverse, then radix-2 DIT with twiddles
     * omega^j; natural order in and out; no 1/n scaling. */
    INIT();
    size_t n = (size_t)1 << log_n;
    for (size_t k = 0; k < n; k++) {
        size_t rk = bitrev(k, log_n);
        if (k < rk) {
            orc_fr t = a[k];
            a[k] = a[rk];
            a[rk] = t;
        }
    }
    if (n < 2) return;
    orc_fr *tw = (orc_fr *)malloc(sizeof(orc_fr) * (n / 2));
    tw_ctx tc = {tw, omega, n / 2, threads};
    parallel_for(n / 2, threads, tw_range, &tc);
    for (unsigned s = 0; s < log_n; s++) {
        fft_ctx c = {a, tw, n, log_n, s};
        parallel_for(n / 2, n >= 4096 ? threads : 1, fft_stage_range, &c);
    }
    free(tw);
}

void orc_fr_omega(orc_fr *out, uint32_t k)
{
    INIT();
    *out = FR_CONST[2];
    for (uint32_t i = k; i < 32; i++) f_mul(out->l, out->l, out->l, &FR);
}

static void scale_all(orc_fr *a, size_t n, const u64 *s)
{
    for (size_t i = 0; i < n; i++) f_mul(a[i].l, a[i].l, s, &FR);
}

void orc_fr_ntt(orc_fr *a, uint32_t log_n, int inverse, int threads)
{
    /* .cu:6488-6502 via sppark NTT: the inverse includes the 1/n factor */
    INIT();
    orc_fr w;
    orc_fr_omega(&w, log_n);
    if (inverse) f_inv(w.l, w.l, &FR);
    orc_fr_fft(a, log_n, &w, threads);
    if (inverse) {
        orc_fr ninv;
        orc_fr_from_u64(&ninv, (uint64_t)1 << log_n);
        f_inv(ninv.l, ninv.l, &FR);
        scale_all(a, (size_t)1 << log_n, ninv.l);
    }
}

void orc_fr_mul_assign_zeta(orc_fr *a, const orc_fr *first, const orc_fr *second, size_t len)
{
    /* domain.rs:551-577 distribute_powers_zeta; .cu:1196-1211 */
    INIT();
    for (size_t i = 0; i < len; i++) {
        size_t k = i % 3;
        if (k == 1) f_mul(a[i].l, a[i].l, first->l, &FR);
        else if (k == 2) f_mul(a[i].l, a[i].l, second->l, &FR);
    }
}

void orc_fr_mul_assign(orc_fr *a, const orc_fr *s, size_t len)
{
    INIT();
    scale_all(a, len, s->l);
}

void orc_fr_mul_assign_repeating(orc_fr *a, const orc_fr *f, size_t flen, size_t len)
{
    /* domain.rs:476-506 divide_by_vanishing_poly; .cu:1213-1223 */
    INIT();
    for (size_t i = 0; i < len; i++) f_mul(a[i].l, a[i].l, f[i % flen].l, &FR);
}

void orc_fr_ntt_zeta(orc_fr *a, uint32_t log_n, int inverse, const orc_fr *scale,
                     const orc_fr *first, const orc_fr *second, int threads)
{
    /* .cu:3447-3495: NTT, then fr_ntt_zeta_postprocess (.cu:1680-1700) */
    INIT();
    if (log_n == 0) return;
    size_t n = (size_t)1 << log_n;
    orc_fr_ntt(a, log_n, inverse, threads);
    scale_all(a, n, scale->l);
    orc_fr_mul_assign_zeta(a, first, second, n);
}

void orc_fr_divide_ntt_zeta(orc_fr *a, uint32_t log_n, const orc_fr *factors, size_t m,
                            const orc_fr *scale, const orc_fr *first, const orc_fr *second,
                            int threads)
{
    /* .cu:3497-3556 */
    INIT();
    if (log_n == 0 || m == 0) return;
    size_t n = (size_t)1 << log_n;
    orc_fr_mul_assign_repeating(a, factors, m, n);
    orc_fr_ntt(a, log_n, 1, threads);
    scale_all(a, n, scale->l);
    orc_fr_mul_assign_zeta(a, first, second, n);
}

int orc_fr_coeff_to_extended_batch(orc_fr *out, const orc_fr *in, size_t input_len, size_t count,
                                   uint32_t ext_log_n, const orc_fr *first, const orc_fr *second,
                                   int threads)
{
    /* domain.rs:325-339 coeff_to_extended; .cu:2542-2602 + prepare kernel
     * .cu:1648-1678: zeta-distribute, zero-pad to 2^ext_log_n, forward NTT */
    INIT();
    size_t out_len = (size_t)1 << ext_log_n;
    if (input_len == 0 || count == 0) return 0;
    if (input_len > out_len) return -1;
    for (size_t p = 0; p < count; p++) {
        orc_fr *o = out + p * out_len;
        memcpy(o, in + p * input_len, sizeof(orc_fr) * input_len);
        memset(o + input_len, 0, sizeof(orc_fr) * (out_len - input_len));
        orc_fr_mul_assign_zeta(o, first, second, input_len);
        orc_fr_ntt(o, ext_log_n, 0, threads);
    }
    return 0;
}

void orc_fr_distribute_powers(orc_fr *a, size_t len, const orc_fr *shift)
{
    /* vendor/sppark-0.1.15/sppark/ntt/kernels.cu:133-153 (LDE_distribute_powers):
     * element i (natural order) times shift^i */
    INIT();
    u64 cur[4];
    memcpy(cur, FR.one, 32);
    for (size_t i = 0; i < len; i++) {
        f_mul(a[i].l, a[i].l, cur, &FR);
        f_mul(cur, cur, shift->l, &FR);
    }
}

void orc_fr_ntt_coset(orc_fr *a, uint32_t log_n, int inverse, const orc_fr *shift, int threads)
{
    /* vendor/sppark-0.1.15/sppark/ntt/ntt.cuh:196-209 (NTT_internal, Type::coset, NN
     * order): the forward transform distributes shift^i before the NTT, the
     * inverse distributes shift^-i after the iNTT (which includes 1/n) */
    INIT();
    if (log_n == 0) return;
    size_t n = (size_t)1 << log_n;
    if (!inverse) {
        orc_fr_distribute_powers(a, n, shift);
        orc_fr_ntt(a, log_n, 0, threads);
    } else {
        orc_fr sinv;
        f_inv(sinv.l, shift->l, &FR);
        orc_fr_ntt(a, log_n, 1, threads);
        orc_fr_distribute_powers(a, n, &sinv);
    }
}

int orc_fr_coeff_to_extended_coset_batch(orc_fr *out, const orc_fr *in, size_t input_len, size_t count,
                                         uint32_t ext_log_n, const orc_fr *shift, int threads)
{
    /* coefficients -> evaluations on shift * <w_ext>: the coset LDE with the
     * coset generator's powers (sppark ntt.cuh:283-338 LDE_aux after its iNTT:
     * LDE_spread_distribute_powers kernels.cu:155-230 multiplies coefficient i
     * by gen^i and spreads it into the zero-padded extended vector, then the
     * forward NTT of the extended domain) */
    INIT();
    size_t out_len = (size_t)1 << ext_log_n;
    if (input_len == 0 || count == 0) return 0;
    if (input_len > out_len) return -1;
    for (size_t p = 0; p < count; p++) {
        orc_fr *o = out + p * out_len;
        memcpy(o, in + p * input_len, sizeof(orc_fr) * input_len);
        memset(o + input_len, 0, sizeof(orc_fr) * (out_len - input_len));
        orc_fr_distribute_powers(o, input_len, shift);
        orc_fr_ntt(o, ext_log_n, 0, threads);
    }
    return 0;
}

void orc_fr_lde_coset(orc_fr *out, const orc_fr *in, uint32_t lg_dsz, uint32_t lg_blowup, int threads)
{
    /* vendor/sppark-0.1.15/sppark/ntt/ntt.cuh:283-338 (NTT::LDE): evaluations on
     * the 2^lg_dsz domain -> coefficients (iNTT) -> coset LDE by the group
     * generator (parameters/bls12_381.h:11, group_gen = 7 = fq.rs GENERATOR) */
    INIT();
    size_t n = (size_t)1 << lg_dsz;
    orc_fr *coeffs = (orc_fr *)malloc(sizeof(orc_fr) * n);
    memcpy(coeffs, in, sizeof(orc_fr) * n);
    orc_fr_ntt(coeffs, lg_dsz, 1, threads);
    orc_fr_coeff_to_extended_coset_batch(out, coeffs, n, 1, lg_dsz + lg_blowup, &FR_CONST[1], threads);
    free(coeffs);
}

uint32_t orc_domain_extended_k(uint32_t j, uint32_t k)
{
    /* domain.rs:56-68 */
    uint64_t n = (uint64_t)1 << k, qd = j - 1;
    uint32_t ek = k;
    while (((uint64_t)1 << ek) < n * qd) ek++;
    return ek;
}

void orc_domain_t_evaluations(orc_fr *out, uint32_t j, uint32_t k)
{
    /* domain.rs:90-124: t(zeta * ext_omega^i) - 1 for i < 2^(ext_k - k), inverted */
    INIT();
    uint32_t ek = orc_domain_extended_k(j, k);
    size_t cnt = (size_t)1 << (ek - k);
    orc_fr ext_w, orig, step, cur;
    orc_fr_omega(&ext_w, ek);
    u64 nexp[1] = {(u64)1 << k};
    f_pow(orig.l, FR_CONST[5].l, nexp, 1, &FR);
    f_pow(step.l, ext_w.l, nexp, 1, &FR);
    cur = orig;
    for (size_t i = 0; i < cnt; i++) {
        f_sub(out[i].l, cur.l, FR.one, &FR);
        f_mul(cur.l, cur.l, step.l, &FR);
    }
    orc_fr_batch_invert(out, cnt);
}

/* ======================================================================== */
/* Grand products and vector ops                                             */
/* ======================================================================== */

void orc_fr_batch_invert(orc_fr *a, size_t len)
{
    /* ff::BatchInvert: Montgomery's trick; zeros are left as zero */
    INIT();
    if (!len) return;
    u64 *pref = (u64 *)malloc(32 * len);
    u64 acc[4];
    memcpy(acc, FR.one, 32);
    for (size_t i = 0; i < len; i++) {
        memcpy(pref + 4 * i, acc, 32);
        if (!mp_is_zero(a[i].l, 4)) f_mul(acc, acc, a[i].l, &FR);
    }
    u64 inv[4];
    f_inv(inv, acc, &FR);
    for (size_t k = len; k-- > 0;) {
        if (mp_is_zero(a[k].l, 4)) continue;
        u64 t[4];
        f_mul(t, inv, pref + 4 * k, &FR);
        f_mul(inv, inv, a[k].l, &FR);
        memcpy(a[k].l, t, 32);
    }
    free(pref);
}

void orc_fr_shifted_prefix_product(orc_fr *values, const orc_fr *initial, size_t len)
{
    /* permutation/prover.rs:36-43: z[0] = initial, z[i] = z[i-1] * v[i-1] */
    INIT();
    if (!len) return;
    u64 prev_v[4], z[4];
    memcpy(z, initial->l, 32);
    memcpy(prev_v, values[0].l, 32);
    memcpy(values[0].l, z, 32);
    for (size_t i = 1; i < len; i++) {
        u64 cur_v[4];
        memcpy(cur_v, values[i].l, 32);
        f_mul(z, z, prev_v, &FR);
        memcpy(values[i].l, z, 32);
        memcpy(prev_v, cur_v, 32);
    }
}

int orc_fr_permutation_products(orc_fr *out, const orc_fr *columns, const orc_fr *permutations,
                                size_t len, size_t column_count, size_t chunk_len,
                                const orc_fr *beta, const orc_fr *gamma, const orc_fr *omega,
                                const orc_fr *delta_powers, const orc_fr *blinds,
                                size_t blinding_factors)
{
    /* permutation/prover.rs:327-533 (Argument::commit, Lagrange values of each
     * set's z); column c of the flattened list uses delta^c (delta_powers[c]). */
    INIT();
    if (!len || !column_count || !chunk_len || blinding_factors >= len) return -1;
    size_t sets = (column_count + chunk_len - 1) / chunk_len;
    orc_fr *mod = (orc_fr *)malloc(sizeof(orc_fr) * len);
    u64 last_z[4];
    memcpy(last_z, FR.one, 32);
    for (size_t s = 0; s < sets; s++) {
        size_t c0 = s * chunk_len, c1 = c0 + chunk_len < column_count ? c0 + chunk_len : column_count;
        for (size_t i = 0; i < len; i++) memcpy(mod[i].l, FR.one, 32);
        for (size_t c = c0; c < c1; c++) {
            for (size_t i = 0; i < len; i++) {
                u64 t[4];
                f_mul(t, beta->l, permutations[c * len + i].l, &FR);
                f_add(t, t, gamma->l, &FR);
                f_add(t, t, columns[c * len + i].l, &FR);
                f_mul(mod[i].l, mod[i].l, t, &FR);
            }
        }
        orc_fr_batch_invert(mod, len);
        for (size_t c = c0; c < c1; c++) {
            u64 dw[4];
            memcpy(dw, delta_powers[c].l, 32);
            for (size_t i = 0; i < len; i++) {
                u64 t[4];
                f_mul(t, dw, beta->l, &FR);
                f_add(t, t, gamma->l, &FR);
                f_add(t, t, columns[c * len + i].l, &FR);
                f_mul(mod[i].l, mod[i].l, t, &FR);
                f_mul(dw, dw, omega->l, &FR);
            }
        }
        orc_fr init;
        memcpy(init.l, last_z, 32);
        orc_fr_shifted_prefix_product(mod, &init, len);
        for (size_t b = 0; b < blinding_factors; b++) mod[len - blinding_factors + b] = blinds[s * blinding_factors + b];
        memcpy(last_z, mod[len - (blinding_factors + 1)].l, 32);
        memcpy(out + s * len, mod, sizeof(orc_fr) * len);
    }
    free(mod);
    return 0;
}

int orc_fr_lookup_products(orc_fr *out, const orc_fr *ci, const orc_fr *ct, const orc_fr *pi,
                           const orc_fr *pt, size_t len, size_t lookup_count,
                           const orc_fr *beta, const orc_fr *gamma, const orc_fr *blinds,
                           size_t blinding_factors)
{
    /* lookup/prover.rs:1075-1240 (construct_product): z[0] = 1,
     * z[i+1] = z[i] * (A+beta)(S+gamma) / ((A'+beta)(S'+gamma)); blinded tail;
     * same shape as .cu:4451-4548. */
    INIT();
    if (!len || !lookup_count || blinding_factors >= len) return -1;
    orc_fr *f = (orc_fr *)malloc(sizeof(orc_fr) * len);
    for (size_t l = 0; l < lookup_count; l++) {
        for (size_t i = 0; i < len; i++) {
            size_t k = l * len + i;
            u64 a[4], b[4];
            f_add(a, pi[k].l, beta->l, &FR);
            f_add(b, pt[k].l, gamma->l, &FR);
            f_mul(f[i].l, a, b, &FR);
        }
        orc_fr_batch_invert(f, len);
        for (size_t i = 0; i < len; i++) {
            size_t k = l * len + i;
            u64 a[4], b[4];
            f_add(a, ci[k].l, beta->l, &FR);
            f_add(b, ct[k].l, gamma->l, &FR);
            f_mul(a, a, b, &FR);
            f_mul(f[i].l, f[i].l, a, &FR);
        }
        orc_fr one;
        memcpy(one.l, FR.one, 32);
        orc_fr_shifted_prefix_product(f, &one, len);
        for (size_t b = 0; b < blinding_factors; b++) f[len - blinding_factors + b] = blinds[l * blinding_factors + b];
        memcpy(out + l * len, f, sizeof(orc_fr) * len);
    }
    free(f);
    return 0;
}

void orc_fr_poly_lincomb(orc_fr *out, const orc_fr *polys, size_t poly_len, size_t poly_count,
                         const orc_fr *scalars)
{
    /* .cu:1593-1611 */
    INIT();
    for (size_t i = 0; i < poly_len; i++) {
        u64 acc[4] = {0, 0, 0, 0};
        for (size_t p = 0; p < poly_count; p++) {
            u64 t[4];
            f_mul(t, polys[p * poly_len + i].l, scalars[p].l, &FR);
            f_add(acc, acc, t, &FR);
        }
        memcpy(out[i].l, acc, 32);
    }
}

int orc_fr_quotient_pieces(orc_fr *out, const orc_fr *q, size_t qlen, size_t poly_len,
                           size_t piece_count, const orc_fr *blinds, size_t blind_count)
{
    /* vanishing/prover.rs:141-220 split into (n-1)-limbs + blind_quotient_limbs
     * (:304-318), laid out as piece_count polynomials of poly_len = n. */
    INIT();
    if (poly_len < 2 || piece_count < 2 || blind_count != piece_count - 1) return -1;
    if (qlen < (poly_len - 1) * piece_count) return -1;
    for (size_t p = 0; p < piece_count; p++) {
        for (size_t i = 0; i + 1 < poly_len; i++) out[p * poly_len + i] = q[p * (poly_len - 1) + i];
        memset(&out[p * poly_len + poly_len - 1], 0, sizeof(orc_fr));
    }
    for (size_t p = 0; p + 1 < piece_count; p++) {
        out[p * poly_len + poly_len - 1] = blinds[p];
        f_sub(out[(p + 1) * poly_len].l, out[(p + 1) * poly_len].l, blinds[p].l, &FR);
    }
    return 0;
}

static int cmp_canon_qsort(const void *a, const void *b)
{
    return orc_fr_cmp_canonical((const orc_fr *)a, (const orc_fr *)b);
}

void orc_fr_sort_canonical(orc_fr *a, size_t len)
{
    INIT();
    qsort(a, len, sizeof(orc_fr), cmp_canon_qsort);
}

/* ======================================================================== */
/* Quotient numerator                                                        */
/* ======================================================================== */


/* eval_polynomial (vendor/midnight-proofs-0.8.1/src/utils/arithmetic.rs:53-77):
 * Horner from the top coefficient */
void orc_fr_eval_poly(orc_fr *out, const orc_fr *poly, size_t len, const orc_fr *point)
{
    INIT();
    u64 acc[4] = {0, 0, 0, 0};
    for (size_t i = len; i-- > 0;) {
        f_mul(acc, acc, point->l, &FR);
        f_add(acc, acc, poly[i].l, &FR);
    }
    memcpy(out->l, acc, sizeof acc);
}

/* kate_division (arithmetic.rs:97-116): q = (a - a(b)) / (X - b), len - 1
 * coefficients: q[len-2] = a[len-1], q[i-1] = a[i] + b * q[i] */
void orc_fr_kate_division(orc_fr *q, const orc_fr *a, size_t len, const orc_fr *b)
{
    INIT();
    if (len < 2) return;
    u64 tmp[4] = {0, 0, 0, 0};
    for (size_t i = len - 1; i >= 1; i--) {
        f_add(q[i - 1].l, a[i].l, tmp, &FR);
        f_mul(tmp, q[i - 1].l, b->l, &FR);
    }
}

/* get_rotation_idx (evaluation.rs:40-45) */
static size_t rot_idx(size_t idx, int32_t rot, int32_t scale, size_t len)
{
    long long v = (long long)idx + (long long)rot * (long long)scale;
    long long m = (long long)len;
    v %= m;
    if (v < 0) v += m;
    return (size_t)v;
}

typedef struct {
    size_t len;
    int32_t rot_scale;
    const orc_fr *fixed, *advice, *instance, *challenges;
    size_t fixed_cols, advice_cols, instance_cols, challenge_len;
    const orc_fr *beta, *gamma, *theta, *trash, *y;
} num_env;

static const orc_fr *col_base(const num_env *e, uint32_t kind, uint32_t index)
{
    if (kind == 0 && index < e->fixed_cols) return e->fixed + (size_t)index * e->len;
    if (kind == 1 && index < e->advice_cols) return e->advice + (size_t)index * e->len;
    if (kind == 2 && index < e->instance_cols) return e->instance + (size_t)index * e->len;
    return NULL;
}

/* ValueSource::get (evaluation.rs:83-129); unknown references read zero,
 * as the reference's GPU interpreter does (.cu:447-516) */
static void src_val(u64 *o, const orc_value_source *src, const orc_graph *g, const num_env *e, size_t idx,
                    const u64 *inter, uint32_t ninter, const u64 *prev)
{
    memset(o, 0, 32);
    switch (src->kind) {
    case 0: if (src->a < g->constants_len) memcpy(o, g->constants[src->a].l, 32); break;
    case 1: if (src->a < ninter) memcpy(o, inter + 4 * src->a, 32); break;
    case 2: case 3: case 4: {
        const orc_fr *b = col_base(e, src->kind - 2, src->a);
        if (b && src->b < g->rotations_len) memcpy(o, b[rot_idx(idx, g->rotations[src->b], e->rot_scale, e->len)].l, 32);
        break;
    }
    case 5: if (src->a < e->challenge_len) memcpy(o, e->challenges[src->a].l, 32); break;
    case 6: memcpy(o, e->beta->l, 32); break;
    case 7: memcpy(o, e->gamma->l, 32); break;
    case 8: memcpy(o, e->theta->l, 32); break;
    case 9: memcpy(o, e->trash->l, 32); break;
    case 10: memcpy(o, e->y->l, 32); break;
    case 11: memcpy(o, prev, 32); break;
    default: break;
    }
}

/* GraphEvaluator::evaluate (evaluation.rs:3797-3846) */
static void eval_graph(u64 *out, const orc_graph *g, const num_env *e, size_t idx, const u64 *prev, u64 *inter)
{
    uint32_t ni = g->num_intermediates;
    memset(inter, 0, 32 * (size_t)ni);
    u64 last[4] = {0, 0, 0, 0};
    for (size_t c = 0; c < g->calculations_len; c++) {
        const orc_calculation *cl = &g->calculations[c];
        u64 a[4], b[4], v[4] = {0, 0, 0, 0};
        switch (cl->op) {
        case 0: src_val(a, &cl->lhs, g, e, idx, inter, ni, prev); src_val(b, &cl->rhs, g, e, idx, inter, ni, prev); f_add(v, a, b, &FR); break;
        case 1: src_val(a, &cl->lhs, g, e, idx, inter, ni, prev); src_val(b, &cl->rhs, g, e, idx, inter, ni, prev); f_sub(v, a, b, &FR); break;
        case 2: src_val(a, &cl->lhs, g, e, idx, inter, ni, prev); src_val(b, &cl->rhs, g, e, idx, inter, ni, prev); f_mul(v, a, b, &FR); break;
        case 3: src_val(a, &cl->lhs, g, e, idx, inter, ni, prev); f_mul(v, a, a, &FR); break;
        case 4: src_val(a, &cl->lhs, g, e, idx, inter, ni, prev); f_add(v, a, a, &FR); break;
        case 5: src_val(a, &cl->lhs, g, e, idx, inter, ni, prev); f_neg(v, a, &FR); break;
        case 6: {
            u64 factor[4];
            src_val(factor, &cl->rhs, g, e, idx, inter, ni, prev);
            src_val(v, &cl->lhs, g, e, idx, inter, ni, prev);
            for (uint32_t k = 0; k < cl->parts_len; k++) {
                u64 part[4] = {0, 0, 0, 0};
                size_t pi = (size_t)cl->parts_offset + k;
                if (pi < g->horner_parts_len) src_val(part, &g->horner_parts[pi], g, e, idx, inter, ni, prev);
                f_mul(v, v, factor, &FR);
                f_add(v, v, part, &FR);
            }
            break;
        }
        case 7: src_val(v, &cl->lhs, g, e, idx, inter, ni, prev); break;
        default: break;
        }
        if (cl->target < ni) memcpy(inter + 4 * cl->target, v, 32);
        memcpy(last, v, 32);
    }
    memcpy(out, last, 32);
}

typedef struct {
    orc_fr *out;
    const orc_fr *initial;
    uint32_t run_custom;
    num_env env;
    const orc_fr *omega, *delta_start, *delta_const;
    int32_t last_rotation;
    uint32_t chunk_len;
    const orc_fr *l0, *l_last, *l_active, *perm_products;
    size_t perm_sets;
    const orc_column_ref *perm_columns;
    size_t perm_columns_len;
    const orc_fr *perm_pk;
    const orc_fr *lk_product, *lk_input, *lk_table;
    size_t lookup_count;
    const orc_fr *trash_cosets;
    const uint32_t *trash_sel;
    size_t trash_count;
    const orc_graph *custom, *lookup_graphs, *trash_graphs;
    uint32_t max_inter;
} num_ctx;

static void num_range(void *vctx, size_t b, size_t e_)
{
    num_ctx *c = (num_ctx *)vctx;
    const num_env *e = &c->env;
    const size_t len = e->len;
    u64 *inter = (u64 *)calloc((size_t)(c->max_inter ? c->max_inter : 1) * 4, sizeof(u64));
    const u64 *one = FR.one;
    u64 zero[4] = {0, 0, 0, 0};
    for (size_t idx = b; idx < e_; idx++) {
        u64 value[4], t[4], t2[4];
        if (c->run_custom) eval_graph(value, c->custom, e, idx, zero, inter);
        else memcpy(value, c->initial[idx].l, 32);
        if (c->perm_sets && c->chunk_len) {
            /* evaluation.rs:3282-3352 */
            size_t r_next = rot_idx(idx, 1, e->rot_scale, len);
            size_t r_last = rot_idx(idx, c->last_rotation, e->rot_scale, len);
            const orc_fr *first = c->perm_products, *last = c->perm_products + (c->perm_sets - 1) * len;
            f_mul(value, value, e->y->l, &FR);
            f_sub(t, one, first[idx].l, &FR);
            f_mul(t, t, c->l0[idx].l, &FR);
            f_add(value, value, t, &FR);
            f_mul(value, value, e->y->l, &FR);
            f_mul(t, last[idx].l, last[idx].l, &FR);
            f_sub(t, t, last[idx].l, &FR);
            f_mul(t, t, c->l_last[idx].l, &FR);
            f_add(value, value, t, &FR);
            for (size_t s = 1; s < c->perm_sets; s++) {
                f_mul(value, value, e->y->l, &FR);
                f_sub(t, c->perm_products[s * len + idx].l, c->perm_products[(s - 1) * len + r_last].l, &FR);
                f_mul(t, t, c->l0[idx].l, &FR);
                f_add(value, value, t, &FR);
            }
            u64 delta[4], wi[4];
            u64 ie[1] = {idx};
            f_pow(wi, c->omega->l, ie, 1, &FR);
            f_mul(delta, c->delta_start->l, wi, &FR);
            for (size_t s = 0; s < c->perm_sets; s++) {
                const orc_fr *prod = c->perm_products + s * len;
                u64 left[4], right[4];
                memcpy(left, prod[r_next].l, 32);
                memcpy(right, prod[idx].l, 32);
                size_t base = s * c->chunk_len;
                for (uint32_t j = 0; j < c->chunk_len && base + j < c->perm_columns_len; j++) {
                    const orc_fr *col = col_base(e, c->perm_columns[base + j].kind, c->perm_columns[base + j].index);
                    if (!col) continue;
                    f_mul(t, e->beta->l, c->perm_pk[(base + j) * len + idx].l, &FR);
                    f_add(t, t, col[idx].l, &FR);
                    f_add(t, t, e->gamma->l, &FR);
                    f_mul(left, left, t, &FR);
                    f_add(t, col[idx].l, delta, &FR);
                    f_add(t, t, e->gamma->l, &FR);
                    f_mul(right, right, t, &FR);
                    f_mul(delta, delta, c->delta_const->l, &FR);
                }
                f_mul(value, value, e->y->l, &FR);
                f_sub(t, left, right, &FR);
                f_mul(t, t, c->l_active[idx].l, &FR);
                f_add(value, value, t, &FR);
            }
        }
        for (size_t n = 0; n < c->lookup_count; n++) {
            /* evaluation.rs:3408-3472 */
            size_t r_next = rot_idx(idx, 1, e->rot_scale, len);
            size_t r_prev = rot_idx(idx, -1, e->rot_scale, len);
            const orc_fr *prod = c->lk_product + n * len, *pin = c->lk_input + n * len, *ptab = c->lk_table + n * len;
            u64 table[4], ams[4];
            eval_graph(table, &c->lookup_graphs[n], e, idx, zero, inter);
            f_sub(ams, pin[idx].l, ptab[idx].l, &FR);
            f_mul(value, value, e->y->l, &FR);
            f_sub(t, one, prod[idx].l, &FR);
            f_mul(t, t, c->l0[idx].l, &FR);
            f_add(value, value, t, &FR);
            f_mul(value, value, e->y->l, &FR);
            f_mul(t, prod[idx].l, prod[idx].l, &FR);
            f_sub(t, t, prod[idx].l, &FR);
            f_mul(t, t, c->l_last[idx].l, &FR);
            f_add(value, value, t, &FR);
            f_mul(value, value, e->y->l, &FR);
            f_add(t, pin[idx].l, e->beta->l, &FR);
            f_mul(t, prod[r_next].l, t, &FR);
            f_add(t2, ptab[idx].l, e->gamma->l, &FR);
            f_mul(t, t, t2, &FR);
            f_mul(t2, prod[idx].l, table, &FR);
            f_sub(t, t, t2, &FR);
            f_mul(t, t, c->l_active[idx].l, &FR);
            f_add(value, value, t, &FR);
            f_mul(value, value, e->y->l, &FR);
            f_mul(t, ams, c->l0[idx].l, &FR);
            f_add(value, value, t, &FR);
            f_mul(value, value, e->y->l, &FR);
            f_sub(t, pin[idx].l, pin[r_prev].l, &FR);
            f_mul(t, ams, t, &FR);
            f_mul(t, t, c->l_active[idx].l, &FR);
            f_add(value, value, t, &FR);
        }
        for (size_t n = 0; n < c->trash_count; n++) {
            /* evaluation.rs:3489-3521 */
            uint32_t sel = c->trash_sel[n];
            if (sel >= e->fixed_cols) continue;
            u64 comp[4];
            eval_graph(comp, &c->trash_graphs[n], e, idx, zero, inter);
            f_sub(t, one, e->fixed[(size_t)sel * len + idx].l, &FR);
            f_mul(t, t, c->trash_cosets[n * len + idx].l, &FR);
            f_sub(t, comp, t, &FR);
            f_mul(value, value, e->y->l, &FR);
            f_add(value, value, t, &FR);
        }
        memcpy(c->out[idx].l, value, 32);
    }
    free(inter);
}

int orc_eval_numerator(orc_fr *out, size_t len, const orc_fr *initial_out, uint32_t run_custom,
                       const orc_fr *fixed, size_t fixed_cols, const orc_fr *advice, size_t advice_cols,
                       const orc_fr *instance, size_t instance_cols, const orc_fr *challenges,
                       size_t challenge_len, const orc_fr *beta, const orc_fr *gamma, const orc_fr *theta,
                       const orc_fr *trash_challenge, const orc_fr *y, const orc_fr *omega,
                       const orc_fr *delta_start, const orc_fr *delta_const, int32_t rot_scale,
                       int32_t last_rotation, uint32_t chunk_len, const orc_fr *l0, const orc_fr *l_last,
                       const orc_fr *l_active, const orc_fr *permutation_products, size_t permutation_sets,
                       const orc_column_ref *permutation_columns, size_t permutation_columns_len,
                       const orc_fr *permutation_pk_cosets, const orc_fr *lookup_product_cosets,
                       const orc_fr *lookup_input_cosets, const orc_fr *lookup_table_cosets,
                       size_t lookup_count, const orc_fr *trash_cosets,
                       const uint32_t *trash_selector_fixed_indices, size_t trash_count,
                       const orc_graph *custom_graph, const orc_graph *lookup_graphs,
                       const orc_graph *trash_graphs, int threads)
{
    INIT();
    if (len == 0) return 0;
    if (!run_custom && !initial_out) return -1;
    num_ctx c;
    memset(&c, 0, sizeof(c));
    c.out = out;
    c.initial = initial_out;
    c.run_custom = run_custom;
    c.env.len = len;
    c.env.rot_scale = rot_scale;
    c.env.fixed = fixed;
    c.env.fixed_cols = fixed_cols;
    c.env.advice = advice;
    c.env.advice_cols = advice_cols;
    c.env.instance = instance;
    c.env.instance_cols = instance_cols;
    c.env.challenges = challenges;
    c.env.challenge_len = challenge_len;
    c.env.beta = beta;
    c.env.gamma = gamma;
    c.env.theta = theta;
    c.env.trash = trash_challenge;
    c.env.y = y;
    c.omega = omega;
    c.delta_start = delta_start;
    c.delta_const = delta_const;
    c.last_rotation = last_rotation;
    c.chunk_len = chunk_len;
    c.l0 = l0;
    c.l_last = l_last;
    c.l_active = l_active;
    c.perm_products = permutation_products;
    c.perm_sets = permutation_sets;
    c.perm_columns = permutation_columns;
    c.perm_columns_len = permutation_columns_len;
    c.perm_pk = permutation_pk_cosets;
    c.lk_product = lookup_product_cosets;
    c.lk_input = lookup_input_cosets;
    c.lk_table = lookup_table_cosets;
    c.lookup_count = lookup_count;
    c.trash_cosets = trash_cosets;
    c.trash_sel = trash_selector_fixed_indices;
    c.trash_count = trash_count;
    c.custom = custom_graph;
    c.lookup_graphs = lookup_graphs;
    c.trash_graphs = trash_graphs;
    uint32_t mx = run_custom ? custom_graph->num_intermediates : 0;
    for (size_t i = 0; i < lookup_count; i++)
        if (lookup_graphs[i].num_intermediates > mx) mx = lookup_graphs[i].num_intermediates;
    for (size_t i = 0; i < trash_count; i++)
        if (trash_graphs[i].num_intermediates > mx) mx = trash_graphs[i].num_intermediates;
    c.max_inter = mx;
    parallel_for(len, threads, num_range, &c);
    return 0;
}

/* ======================================================================== */
/* BLAKE2b (RFC 7693), for the transcript checks                            */
/* ======================================================================== */

typedef struct {
    u64 h[8], t[2];
    uint8_t b[128];
    size_t c, outlen;
} b2b_ctx;

static const u64 B2B_IV[8] = {0x6a09e667f3bcc908ULL, 0xbb67ae8584caa73bULL, 0x3c6ef372fe94f82bULL,
                              0xa54ff53a5f1d36f1ULL, 0x510e527fade682d1ULL, 0x9b05688c2b3e6c1fULL,
                              0x1f83d9abfb41bd6bULL, 0x5be0cd19137e2179ULL};
static const uint8_t B2B_SIGMA[12][16] = {
    {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15}, {14, 10, 4, 8, 9, 15, 13, 6, 1, 12, 0, 2, 11, 7, 5, 3},
    {11, 8, 12, 0, 5, 2, 15, 13, 10, 14, 3, 6, 7, 1, 9, 4}, {7, 9, 3, 1, 13, 12, 11, 14, 2, 6, 5, 10, 4, 0, 15, 8},
    {9, 0, 5, 7, 2, 4, 10, 15, 14, 1, 11, 12, 6, 8, 3, 13}, {2, 12, 6, 10, 0, 11, 8, 3, 4, 13, 7, 5, 15, 14, 1, 9},
    {12, 5, 1, 15, 14, 13, 4, 10, 0, 7, 6, 3, 9, 2, 8, 11}, {13, 11, 7, 14, 12, 1, 3, 9, 5, 0, 15, 4, 8, 6, 2, 10},
    {6, 15, 14, 9, 11, 3, 0, 8, 12, 2, 13, 7, 1, 4, 10, 5}, {10, 2, 8, 4, 7, 6, 1, 5, 15, 11, 9, 14, 3, 12, 13, 0},
    {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15}, {14, 10, 4, 8, 9, 15, 13, 6, 1, 12, 0, 2, 11, 7, 5, 3}};

static u64 rotr64(u64 x, int n) { return (x >> n) | (x << (64 - n)); }

static void b2b_compress(b2b_ctx *ctx, int last)
{
    u64 v[16], m[16];
    for (int i = 0; i < 8; i++) {
        v[i] = ctx->h[i];
        v[i + 8] = B2B_IV[i];
    }
    v[12] ^= ctx->t[0];
    v[13] ^= ctx->t[1];
    if (last) v[14] = ~v[14];
    for (int i = 0; i < 16; i++) {
        m[i] = 0;
        for (int k = 0; k < 8; k++) m[i] |= (u64)ctx->b[8 * i + k] << (8 * k);
    }
#define B2B_G(a, b, c, d, x, y)                \
    do {                                       \
        v[a] = v[a] + v[b] + (x);              \
        v[d] = rotr64(v[d] ^ v[a], 32);        \
        v[c] = v[c] + v[d];                    \
        v[b] = rotr64(v[b] ^ v[c], 24);        \
        v[a] = v[a] + v[b] + (y);              \
        v[d] = rotr64(v[d] ^ v[a], 16);        \
        v[c] = v[c] + v[d];                    \
        v[b] = rotr64(v[b] ^ v[c], 63);        \
    } while (0)
    for (int r = 0; r < 12; r++) {
        const uint8_t *s = B2B_SIGMA[r];
        B2B_G(0, 4, 8, 12, m[s[0]], m[s[1]]);
        B2B_G(1, 5, 9, 13, m[s[2]], m[s[3]]);
        B2B_G(2, 6, 10, 14, m[s[4]], m[s[5]]);
        B2B_G(3, 7, 11, 15, m[s[6]], m[s[7]]);
        B2B_G(0, 5, 10, 15, m[s[8]], m[s[9]]);
        B2B_G(1, 6, 11, 12, m[s[10]], m[s[11]]);
        B2B_G(2, 7, 8, 13, m[s[12]], m[s[13]]);
        B2B_G(3, 4, 9, 14, m[s[14]], m[s[15]]);
    }
#undef B2B_G
    for (int i = 0; i < 8; i++) ctx->h[i] ^= v[i] ^ v[i + 8];
}

static void b2b_update(b2b_ctx *ctx, const uint8_t *in, size_t len)
{
    for (size_t i = 0; i < len; i++) {
        if (ctx->c == 128) {
            ctx->t[0] += ctx->c;
            if (ctx->t[0] < ctx->c) ctx->t[1]++;
            b2b_compress(ctx, 0);
            ctx->c = 0;
        }
        ctx->b[ctx->c++] = in[i];
    }
}

static void b2b_init(b2b_ctx *ctx, size_t outlen, const uint8_t *key, size_t keylen)
{
    for (int i = 0; i < 8; i++) ctx->h[i] = B2B_IV[i];
    ctx->h[0] ^= 0x01010000ULL ^ ((u64)keylen << 8) ^ (u64)outlen;
    ctx->t[0] = ctx->t[1] = 0;
    ctx->c = 0;
    ctx->outlen = outlen;
    memset(ctx->b, 0, 128);
    if (keylen) {
        b2b_update(ctx, key, keylen);
        ctx->c = 128;
    }
}

/* digest of the state so far, leaving the state usable (like
 * blake2b_simd::State::finalize, which works on a copy) */
static void b2b_final_copy(const b2b_ctx *in, uint8_t *out)
{
    b2b_ctx ctx = *in;
    ctx.t[0] += ctx.c;
    if (ctx.t[0] < ctx.c) ctx.t[1]++;
    while (ctx.c < 128) ctx.b[ctx.c++] = 0;
    b2b_compress(&ctx, 1);
    for (size_t i = 0; i < ctx.outlen; i++) out[i] = (uint8_t)(ctx.h[i >> 3] >> (8 * (i & 7)));
}

void orc_blake2b(uint8_t *out, size_t outlen, const uint8_t *key, size_t keylen, const uint8_t *in, size_t len)
{
    b2b_ctx ctx;
    b2b_init(&ctx, outlen, key, keylen);
    b2b_update(&ctx, in, len);
    b2b_final_copy(&ctx, out);
}

/* Transcript replay (transcript/mod.rs:95-150, implementors.rs:13-33):
 * ops[i] = 1 absorbs msgs[i] (prefix 0x01), ops[i] = 0 squeezes (prefix 0x00
 * then digest -> from_uniform_bytes) into challenges[j++]. */
void orc_transcript_replay(const uint8_t *ops, size_t nops, const uint8_t *const *msgs, const size_t *lens,
                           orc_fr *challenges)
{
    INIT();
    static const uint8_t key[] = "Domain separator for transcript";
    b2b_ctx ctx;
    b2b_init(&ctx, 64, key, sizeof(key) - 1);
    size_t j = 0;
    for (size_t i = 0; i < nops; i++) {
        if (ops[i]) {
            uint8_t one = 1;
            b2b_update(&ctx, &one, 1);
            b2b_update(&ctx, msgs[i], lens[i]);
        } else {
            uint8_t zero = 0, d[64];
            b2b_update(&ctx, &zero, 1);
            b2b_final_copy(&ctx, d);
            orc_fr_from_uniform_bytes(&challenges[j++], d);
        }
    }
}
