/*
 * orc_rng.c -- MRG32k3a with streams and substreams (RngStream restated).
 *
 * TEST INFRASTRUCTURE ONLY (the oracle; see ffea_oracle.h).
 *
 * Restates the published generator of L'Ecuyer (Operations Research 47(1),
 * 1999) with the stream/substream package of L'Ecuyer, Simard, Chen and
 * Kelton (Operations Research 50(6), 2002), as vendored by the reference in
 * src/RngStream.cpp. The reference keeps the state in doubles holding exact
 * integers; this file keeps it in uint32 and does exact modular arithmetic in
 * 64 bits, which yields the same integer states. The floating-point outputs
 * are formed exactly as the reference forms them:
 *   U01          src/RngStream.cpp:266-289
 *   U01d         :294-309 (increased precision)
 *   RandU01      :509-515, RandInt :519-522
 *   streams      ctor :327-345 (next seed advanced by A^(2^127))
 *   substreams   ResetNextSubstream :371-378 (A^(2^76))
 *   AdvanceState :408-435 (2^e + c steps, negative = backwards)
 *   SetPackageSeed / CheckSeed :381-389, :225-262
 * The jump matrices are computed here from the recurrence coefficients by
 * repeated squaring instead of being tabulated.
 */
#include "ffea_oracle.h"

#include <stdlib.h>

#define M1 4294967087ULL
#define M2 4294944443ULL
#define A12 1403580ULL
#define A13N 810728ULL
#define A21 527612ULL
#define A23N 1370589ULL

typedef uint64_t mat3u[3][3];

static uint64_t mulmod(uint64_t a, uint64_t b, uint64_t m) { return (a % m) * (b % m) % m; }

static void matmat(const mat3u A, const mat3u B, mat3u C, uint64_t m) {
    mat3u W;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            uint64_t s = 0;
            for (int k = 0; k < 3; ++k) s = (s + mulmod(A[i][k], B[k][j], m)) % m;
            W[i][j] = s;
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) C[i][j] = W[i][j];
}

static void matvec(const mat3u A, uint32_t *s, uint64_t m) {
    uint64_t x[3];
    for (int i = 0; i < 3; ++i) {
        uint64_t t = 0;
        for (int k = 0; k < 3; ++k) t = (t + mulmod(A[i][k], s[k], m)) % m;
        x[i] = t;
    }
    for (int i = 0; i < 3; ++i) s[i] = (uint32_t)x[i];
}

static void matpow(const mat3u A, uint64_t n, mat3u B, uint64_t m) {
    mat3u W;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) { W[i][j] = A[i][j]; B[i][j] = (i == j); }
    while (n) {
        if (n & 1) matmat(W, B, B, m);
        matmat(W, W, W, m);
        n >>= 1;
    }
}

static void mattwopow(const mat3u A, int e, mat3u B, uint64_t m) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) B[i][j] = A[i][j];
    for (int i = 0; i < e; ++i) matmat(B, B, B, m);
}

/* modular inverse by the extended Euclidean algorithm */
static uint64_t invmod(uint64_t a, uint64_t m) {
    int64_t t = 0, nt = 1, r = (int64_t)m, nr = (int64_t)(a % m);
    while (nr) {
        int64_t q = r / nr, tmp;
        tmp = t - q * nt; t = nt; nt = tmp;
        tmp = r - q * nr; r = nr; nr = tmp;
    }
    if (t < 0) t += (int64_t)m;
    return (uint64_t)t;
}

/* one-step transition matrices of the two components and their inverses */
static mat3u A1, A2, A1inv, A2inv, A1p76, A2p76, A1p127, A2p127;
static int tables_ready = 0;

static void init_tables(void) {
    if (tables_ready) return;
    mat3u a1 = {{0, 1, 0}, {0, 0, 1}, {M1 - A13N, A12, 0}};
    mat3u a2 = {{0, 1, 0}, {0, 0, 1}, {M2 - A23N, 0, A21}};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) { A1[i][j] = a1[i][j]; A2[i][j] = a2[i][j]; }
    /* x_{n-4} = (a12 x_{n-3} - x_{n-1}) / a13n  (component 1)
       x_{n-4} = (a21 x_{n-2} - x_{n-1}) / a23n  (component 2) */
    uint64_t i13 = invmod(A13N, M1), i23 = invmod(A23N, M2);
    mat3u b1 = {{mulmod(A12, i13, M1), 0, (M1 - i13) % M1}, {1, 0, 0}, {0, 1, 0}};
    mat3u b2 = {{0, mulmod(A21, i23, M2), (M2 - i23) % M2}, {1, 0, 0}, {0, 1, 0}};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) { A1inv[i][j] = b1[i][j]; A2inv[i][j] = b2[i][j]; }
    mattwopow(A1, 76, A1p76, M1);
    mattwopow(A2, 76, A2p76, M2);
    mattwopow(A1, 127, A1p127, M1);
    mattwopow(A2, 127, A2p127, M2);
    tables_ready = 1;
}

static uint32_t next_seed[6] = {12345, 12345, 12345, 12345, 12345, 12345};

int orc_rng_check_seed(const uint32_t s[6]) {
    for (int i = 0; i < 3; ++i)
        if (s[i] >= M1) return -1;
    for (int i = 3; i < 6; ++i)
        if (s[i] >= M2) return -1;
    if (s[0] == 0 && s[1] == 0 && s[2] == 0) return -1;
    if (s[3] == 0 && s[4] == 0 && s[5] == 0) return -1;
    return 0;
}

void orc_rng_set_package_seed(const uint32_t seed[6]) {
    if (orc_rng_check_seed(seed)) return;
    for (int i = 0; i < 6; ++i) next_seed[i] = seed[i];
}

void orc_rng_create(orc_rng *g) {
    init_tables();
    g->anti = 0;
    g->inc_prec = 0;
    for (int i = 0; i < 6; ++i) g->Bg[i] = g->Cg[i] = g->Ig[i] = next_seed[i];
    matvec(A1p127, next_seed, M1);
    matvec(A2p127, next_seed + 3, M2);
}

void orc_rng_set_state(orc_rng *g, const uint32_t s[6]) {
    init_tables();
    for (int i = 0; i < 6; ++i) g->Bg[i] = g->Cg[i] = g->Ig[i] = s[i];
}

void orc_rng_get_state(const orc_rng *g, uint32_t out[6]) {
    for (int i = 0; i < 6; ++i) out[i] = g->Cg[i];
}

void orc_rng_reset_start_stream(orc_rng *g) {
    for (int i = 0; i < 6; ++i) g->Cg[i] = g->Bg[i] = g->Ig[i];
}

void orc_rng_reset_start_substream(orc_rng *g) {
    for (int i = 0; i < 6; ++i) g->Cg[i] = g->Bg[i];
}

void orc_rng_reset_next_substream(orc_rng *g) {
    init_tables();
    matvec(A1p76, g->Bg, M1);
    matvec(A2p76, g->Bg + 3, M2);
    for (int i = 0; i < 6; ++i) g->Cg[i] = g->Bg[i];
}

void orc_rng_advance_state(orc_rng *g, int32_t e, int32_t c) {
    init_tables();
    mat3u B1, B2, C1, C2;
    if (e > 0) {
        mattwopow(A1, e, B1, M1);
        mattwopow(A2, e, B2, M2);
    } else if (e < 0) {
        mattwopow(A1inv, -e, B1, M1);
        mattwopow(A2inv, -e, B2, M2);
    }
    if (c >= 0) {
        matpow(A1, (uint64_t)c, C1, M1);
        matpow(A2, (uint64_t)c, C2, M2);
    } else {
        matpow(A1inv, (uint64_t)(-(int64_t)c), C1, M1);
        matpow(A2inv, (uint64_t)(-(int64_t)c), C2, M2);
    }
    if (e) {
        matmat(B1, C1, C1, M1);
        matmat(B2, C2, C2, M2);
    }
    matvec(C1, g->Cg, M1);
    matvec(C2, g->Cg + 3, M2);
}

void orc_rng_set_antithetic(orc_rng *g, int a) { g->anti = a != 0; }
void orc_rng_increased_precis(orc_rng *g, int p) { g->inc_prec = p != 0; }

static double u01(orc_rng *g) {
    uint32_t *s = g->Cg;
    /* component 1: x_n = a12 x_{n-2} - a13n x_{n-3} mod m1 */
    uint64_t p1 = ((A12 * s[1]) % M1 + M1 - (A13N * s[0]) % M1) % M1;
    s[0] = s[1]; s[1] = s[2]; s[2] = (uint32_t)p1;
    /* component 2: x_n = a21 x_{n-1} - a23n x_{n-3} mod m2 */
    uint64_t p2 = ((A21 * s[5]) % M2 + M2 - (A23N * s[3]) % M2) % M2;
    s[3] = s[4]; s[4] = s[5]; s[5] = (uint32_t)p2;
    const double norm = 1.0 / ((double)M1 + 1.0);
    double d1 = (double)p1, d2 = (double)p2;
    double u = (p1 > p2) ? (d1 - d2) * norm : (d1 - d2 + (double)M1) * norm;
    return g->anti ? (1 - u) : u;
}

static double u01d(orc_rng *g) {
    const double fact = 5.9604644775390625e-8; /* 2^-24 */
    double u = u01(g);
    if (g->anti) {
        u += (u01(g) - 1.0) * fact;
        return (u < 0.0) ? u + 1.0 : u;
    }
    u += u01(g) * fact;
    return (u < 1.0) ? u : (u - 1.0);
}

double orc_rng_rand_u01(orc_rng *g) { return g->inc_prec ? u01d(g) : u01(g); }

int orc_rng_rand_int(orc_rng *g, int lo, int hi) {
    return lo + (int)((hi - lo + 1.0) * orc_rng_rand_u01(g));
}

void orc_seed_from_rng_seed(int rng_seed, uint32_t out[6]) {
    const uint32_t two_max[2] = {4294967087u, 4294944443u};
    srand((unsigned)rng_seed);
    for (int i = 0; i < 6; ++i) {
        uint32_t r1 = (uint32_t)rand(), r2 = (uint32_t)rand();
        out[i] = (uint32_t)(r1 + r2) % two_max[i / 3];
    }
}
