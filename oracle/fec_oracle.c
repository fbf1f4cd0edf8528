/*
 * CPU oracle for the receive-side FEC path -- TEST INFRASTRUCTURE ONLY.
 * See fec_oracle.h for what it restates and what pins it.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load this code.
 *
 * Build: oracle/build.py (gcc -O2 -fopenmp -ffp-contract=off -shared).
 */
#include "fec_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../cusat_gb300/csrc/cusat_data.h"
#include "../cusat_gb300/csrc/gen/code_tables.inc"

#define M 360

/* ------------------------------------------------------------------------ */
/* Code structure built from the raw ETSI rows                               */
/* ------------------------------------------------------------------------ */

typedef struct {
    int built, ok;
    int N, K, R, q, cnl, links_total;
    int* lay_off;   /* [q+1] into circ_g/circ_s */
    int* circ_g;    /* info group (row) of each circulant of a layer */
    int* circ_s;    /* shift: check j of the layer uses bit g*360 + (j - s) mod 360 */
    int* msg_off;   /* [q] start of layer i's message block, 360*(cnt+2) bytes */
    int msg_total;
    int n_steps;
    int16_t* sched; /* [n_steps*2] */
    int k_bch, n_bch, t, p;
    uint64_t gen[4];
    const cusat_table_src* src;
} orc_code;

static orc_code g_codes[3][CUSAT_RATE_COUNT];

static int poly_degree(const uint64_t* a)
{
    for (int i = 255; i >= 0; i--)
        if ((a[i >> 6] >> (i & 63)) & 1)
            return i;
    return -1;
}

/* a *= b over GF(2); b has degree < 32. */
static void poly_mul_small(uint64_t* a, uint32_t b)
{
    uint64_t r[4] = {0, 0, 0, 0};
    for (int i = 0; i < 32; i++) {
        if (!((b >> i) & 1))
            continue;
        /* r ^= a << i */
        for (int w = 3; w >= 0; w--) {
            uint64_t v = a[w] << i;
            if (i && w > 0)
                v |= a[w - 1] >> (64 - i);
            r[w] ^= v;
        }
    }
    memcpy(a, r, sizeof(r));
}

static void build_code(orc_code* c, int framesize, int rate)
{
    c->built = 1;
    c->ok = 0;
    const char* name = cusat_table_name(framesize, rate);
    const cusat_bch_row* br = cusat_find_bch_row(framesize, rate);
    if (!name || !br)
        return;
    const cusat_table_src* src = 0;
    for (int i = 0; i < CUSAT_N_TABLE_SRCS; i++)
        if (!strcmp(cusat_table_srcs[i].name, name))
            src = &cusat_table_srcs[i];
    if (!src)
        return;
    c->src = src;
    c->N = src->n;
    c->K = src->k;
    c->R = c->N - c->K;
    c->q = c->R / M;
    c->cnl = src->links_max_cn - 2;
    c->links_total = src->links_total;
    const int q = c->q;
    /* group circulants by layer = address mod q */
    int* cnt = (int*)calloc(q, sizeof(int));
    int n_addr = 0;
    for (int r = 0; r < src->n_rows; r++)
        n_addr += src->row_deg[r];
    const uint16_t* a = src->addr;
    for (int r = 0, o = 0; r < src->n_rows; r++)
        for (int d = 0; d < src->row_deg[r]; d++, o++)
            cnt[a[o] % q]++;
    c->lay_off = (int*)malloc((q + 1) * sizeof(int));
    c->lay_off[0] = 0;
    for (int i = 0; i < q; i++)
        c->lay_off[i + 1] = c->lay_off[i] + cnt[i];
    c->circ_g = (int*)malloc(n_addr * sizeof(int));
    c->circ_s = (int*)malloc(n_addr * sizeof(int));
    int* fill = (int*)calloc(q, sizeof(int));
    for (int r = 0, o = 0; r < src->n_rows; r++)
        for (int d = 0; d < src->row_deg[r]; d++, o++) {
            int i = a[o] % q;
            int k = c->lay_off[i] + fill[i]++;
            c->circ_g[k] = r;
            c->circ_s[k] = a[o] / q;
        }
    c->msg_off = (int*)malloc(q * sizeof(int));
    int tot = 0;
    for (int i = 0; i < q; i++) {
        c->msg_off[i] = tot;
        tot += M * (cnt[i] + 2);
    }
    c->msg_total = tot;
    free(cnt);
    free(fill);
    /* schedule: the paired schedule built for this table, else sequential
     * (reference ldpc_decode_kernel.cu:1121-1170, ldpc_schedule_registry.h:102-106) */
    const cusat_sched_src* ss = 0;
    for (int i = 0; i < CUSAT_N_SCHED_SRCS; i++)
        if (!strcmp(cusat_sched_srcs[i].name, name) && cusat_sched_srcs[i].q == q)
            ss = &cusat_sched_srcs[i];
    if (ss) {
        c->n_steps = ss->n_steps;
        c->sched = (int16_t*)malloc(2 * ss->n_steps * sizeof(int16_t));
        memcpy(c->sched, ss->pairs, 2 * ss->n_steps * sizeof(int16_t));
    } else {
        c->n_steps = q;
        c->sched = (int16_t*)malloc(2 * q * sizeof(int16_t));
        for (int i = 0; i < q; i++) {
            c->sched[2 * i] = (int16_t)i;
            c->sched[2 * i + 1] = -1;
        }
    }
    /* BCH: generator = g1 * g2 * ... * gt (reference fec/bch_code.cc:99-122) */
    c->k_bch = (int)br->k_bch;
    c->n_bch = (int)br->n_bch;
    c->t = (int)br->t;
    memset(c->gen, 0, sizeof(c->gen));
    c->gen[0] = 1;
    int fam = framesize == CUSAT_FECFRAME_NORMAL ? 0 : framesize == CUSAT_FECFRAME_SHORT ? 1 : 2;
    for (int i = 0; i < c->t; i++)
        poly_mul_small(c->gen, cusat_bch_minpoly[fam][i]);
    c->p = poly_degree(c->gen);
    c->ok = (c->p > 0 && c->k_bch == c->n_bch - c->p && c->n_bch == c->K);
}

static const orc_code* get_code(int framesize, int rate)
{
    if (framesize < 0 || framesize > 2 || rate < 0 || rate >= CUSAT_RATE_COUNT)
        return 0;
    orc_code* c = &g_codes[framesize][rate];
#ifdef _OPENMP
#pragma omp critical(orc_build)
#endif
    {
        if (!c->built)
            build_code(c, framesize, rate);
    }
    return c->ok ? c : 0;
}

int orc_code_info(int framesize, int rate, int32_t* out)
{
    const orc_code* c = get_code(framesize, rate);
    if (!c)
        return -1;
    out[0] = c->N;
    out[1] = c->K;
    out[2] = c->q;
    out[3] = c->n_steps;
    out[4] = c->k_bch;
    out[5] = c->n_bch;
    out[6] = c->t;
    out[7] = c->p;
    out[8] = c->links_total;
    out[9] = c->cnl;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Reference arithmetic (ldpc_decode_kernel.cu:32-58, ldpc_message_update.h) */
/* ------------------------------------------------------------------------ */

static inline int16_t qabs(int16_t a) { return (a == -32768) ? 32767 : (a < 0 ? -a : a); }
static inline uint16_t qsubu(uint16_t a, uint16_t b) { return a > b ? (uint16_t)(a - b) : 0; }
static inline int16_t qsign(int16_t a, int16_t b) { return b < 0 ? (int16_t)-a : (b > 0 ? a : 0); }
static inline int16_t qsat16(int v) { return (int16_t)(v < -32768 ? -32768 : (v > 32767 ? 32767 : v)); }
static inline int8_t clamp_bnl(int v) { return (int8_t)(v < -127 ? -127 : (v > 127 ? 127 : v)); }

int orc_bnl_update(int raw_new, int old, int32_t* delta)
{
    int8_t m = clamp_bnl(raw_new);
    *delta = (int)m - old;
    return m;
}

/* nms_scale of ldpc_decode_kernel.cu:75-90 with alpha in 64ths; <= 0 = off */
static inline int nms_scale(int v, int n)
{
    if (n <= 0)
        return v;
    int m = ((v < 0 ? -v : v) * n + 32) >> 6;
    return v < 0 ? -m : m;
}

/* finalp_oms_i16 (ldpc_decode_kernel.cu:242-275) with a runtime beta. */
static void finalp(int16_t* links, int deg, uint16_t beta)
{
    int16_t min1, min2;
    int16_t xs = links[0];
    {
        uint16_t m0 = qsubu((uint16_t)qabs(links[0]), beta);
        uint16_t m1 = qsubu((uint16_t)qabs(links[1]), beta);
        xs ^= links[1];
        if (m0 <= m1) {
            min1 = (int16_t)m0;
            min2 = (int16_t)m1;
        } else {
            min1 = (int16_t)m1;
            min2 = (int16_t)m0;
        }
    }
    for (int i = 2; i < deg; i++) {
        xs ^= links[i];
        int16_t m = (int16_t)qsubu((uint16_t)qabs(links[i]), beta);
        if (m < min1) {
            min2 = min1;
            min1 = m;
        } else if (m < min2) {
            min2 = m;
        }
    }
    for (int i = 0; i < deg; i++) {
        int16_t m = (int16_t)qsubu((uint16_t)qabs(links[i]), beta);
        int16_t oth = (m == min1) ? min2 : min1;
        int16_t s = (int16_t)((xs ^ links[i]) | 0x7FFF);
        links[i] = qsign(oth, s);
    }
}

/* ------------------------------------------------------------------------ */
/* Layered decoder                                                            */
/* ------------------------------------------------------------------------ */

typedef struct {
    int16_t* app_d;  /* [K] */
    int16_t* app_p;  /* [R], transposed: slot i*M + j = parity bit q*j + i */
    int8_t* msg;     /* [msg_total] */
    int32_t* acc;    /* [K] pending deltas of the current step */
    int32_t* stamp;  /* [K] step id of the last delta */
    int32_t* touched;
    int32_t* pslot;  /* pending parity writes */
    int16_t* pval;
} orc_work;

static int syndrome_ok(const orc_code* c, const int16_t* app_d, const int16_t* app_p)
{
    const int q = c->q;
    for (int i = 0; i < q; i++) {
        const int lo = c->lay_off[i], hi = c->lay_off[i + 1];
        for (int j = 0; j < M; j++) {
            int par = (app_p[M * i + j] < 0);
            if (i > 0)
                par ^= (app_p[M * (i - 1) + j] < 0);
            else if (j > 0)
                par ^= (app_p[j + (q - 1) * M - 1] < 0);
            for (int k = lo; k < hi; k++) {
                int s = c->circ_s[k];
                int v = c->circ_g[k] * M + ((j - s + M) % M);
                par ^= (app_d[v] < 0);
            }
            if (par)
                return 0;
        }
    }
    return 1;
}

static void pack_hard(const int16_t* app_d, int K, uint8_t* hard)
{
    for (int b = 0; b < K / 8; b++) {
        uint8_t byte = 0;
        for (int k = 0; k < 8; k++)
            if (app_d[8 * b + k] < 0)
                byte |= (uint8_t)(1 << (7 - k));
        hard[b] = byte;
    }
}

static void decode_frame(const orc_code* c, orc_work* w, const int16_t* llr, int T, int period,
                         const int16_t* weights, uint8_t* hard, int32_t* result)
{
    const int K = c->K, R = c->R, q = c->q;
    /* init (ldpc_decode_kernel.cu:655-670): clamp to +-32767, parity transpose */
    for (int v = 0; v < K; v++) {
        int x = llr[v];
        w->app_d[v] = (int16_t)(x < -32767 ? -32767 : (x > 32767 ? 32767 : x));
    }
    for (int idx = 0; idx < R; idx++) {
        int x = llr[K + idx];
        w->app_p[M * (idx % q) + idx / q] = (int16_t)(x < -32767 ? -32767 : (x > 32767 ? 32767 : x));
    }
    memset(w->msg, 0, c->msg_total);
    memset(w->stamp, 0xff, K * sizeof(int32_t));
    int step_id = 0;
    int16_t x[64];
    int vn[64];
    for (int trial = 0; trial <= T; trial++) {
        /* periodic + final check (ldpc_decode_kernel.cu:693-694) */
        if ((trial % period == 0 || trial == T) && syndrome_ok(c, w->app_d, w->app_p)) {
            pack_hard(w->app_d, K, hard);
            *result = T - trial;
            return;
        }
        if (trial == T)
            break;
        for (int st = 0; st < c->n_steps; st++, step_id++) {
            int n_touched = 0, n_par = 0;
            /* phase A: every check of the step gathers from the step-start state */
            for (int lane = 0; lane < 2; lane++) {
                const int i = c->sched[2 * st + lane];
                if (i < 0)
                    continue;
                const int lo = c->lay_off[i], cnt = c->lay_off[i + 1] - lo;
                for (int j = 0; j < M; j++) {
                    const int deg = cnt + 2 - (i == 0 && j == 0 ? 1 : 0);
                    int8_t* bl = w->msg + c->msg_off[i] + j * (cnt + 2);
                    for (int e = 0; e < cnt; e++) {
                        const int s = c->circ_s[lo + e];
                        vn[e] = c->circ_g[lo + e] * M + ((j - s + M) % M);
                        x[e] = qsat16((int)w->app_d[vn[e]] - (int)bl[e]);
                    }
                    int ps0 = M * i + j, ps1 = -1;
                    x[cnt] = qsat16((int)w->app_p[ps0] - (int)bl[cnt]);
                    if (i > 0)
                        ps1 = M * (i - 1) + j;
                    else if (j > 0)
                        ps1 = j + (q - 1) * M - 1;
                    if (ps1 >= 0)
                        x[cnt + 1] = qsat16((int)w->app_p[ps1] - (int)bl[cnt + 1]);
                    const int16_t xp0 = x[cnt];
                    const int16_t xp1 = ps1 >= 0 ? x[cnt + 1] : 0;
                    uint16_t beta = 1;
                    int alpha = 0;
                    if (weights) {
                        const int16_t* wt = weights + ((size_t)trial * 32 + deg) * 2;
                        beta = (uint16_t)wt[0];
                        alpha = wt[1];
                    }
                    finalp(x, deg, beta);
                    for (int e = 0; e < cnt; e++) {
                        const int8_t m = clamp_bnl(nms_scale(x[e], alpha));
                        const int v = vn[e];
                        if (w->stamp[v] != step_id) {
                            w->stamp[v] = step_id;
                            w->acc[v] = 0;
                            w->touched[n_touched++] = v;
                        }
                        w->acc[v] += (int)m - (int)bl[e];
                        bl[e] = m;
                    }
                    {
                        const int8_t m = clamp_bnl(nms_scale(x[cnt], alpha));
                        w->pslot[n_par] = ps0;
                        w->pval[n_par++] = qsat16((int)xp0 + (int)m);
                        bl[cnt] = m;
                    }
                    if (ps1 >= 0) {
                        const int8_t m = clamp_bnl(nms_scale(x[cnt + 1], alpha));
                        w->pslot[n_par] = ps1;
                        w->pval[n_par++] = qsat16((int)xp1 + (int)m);
                        bl[cnt + 1] = m;
                    }
                }
            }
            /* phase B: apply */
            for (int k = 0; k < n_touched; k++) {
                const int v = w->touched[k];
                w->app_d[v] = qsat16((int)w->app_d[v] + w->acc[v]);
            }
            for (int k = 0; k < n_par; k++)
                w->app_p[w->pslot[k]] = w->pval[k];
        }
    }
    pack_hard(w->app_d, K, hard);
    *result = -1;
}

int orc_ldpc_decode(int framesize, int rate, const int16_t* llr, int B, int max_trials,
                    const int16_t* weights, uint8_t* hard, int32_t* trials, int nthreads)
{
    return orc_ldpc_decode_period(framesize, rate, llr, B, max_trials, 1, weights, hard, trials, nthreads);
}

int orc_ldpc_decode_period(int framesize, int rate, const int16_t* llr, int B, int max_trials, int syn_period,
                           const int16_t* weights, uint8_t* hard, int32_t* trials, int nthreads)
{
    const orc_code* c = get_code(framesize, rate);
    if (!c || B < 0 || max_trials < 0 || syn_period < 1)
        return -1;
    if (nthreads <= 0)
        nthreads = 1;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
    {
        orc_work w;
        w.app_d = (int16_t*)malloc(c->K * sizeof(int16_t));
        w.app_p = (int16_t*)malloc(c->R * sizeof(int16_t));
        w.msg = (int8_t*)malloc(c->msg_total);
        w.acc = (int32_t*)malloc(c->K * sizeof(int32_t));
        w.stamp = (int32_t*)malloc(c->K * sizeof(int32_t));
        w.touched = (int32_t*)malloc(2 * M * 64 * sizeof(int32_t));
        w.pslot = (int32_t*)malloc(4 * M * sizeof(int32_t));
        w.pval = (int16_t*)malloc(4 * M * sizeof(int16_t));
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (int f = 0; f < B; f++)
            decode_frame(c, &w, llr + (size_t)f * c->N, max_trials, syn_period, weights,
                         hard + (size_t)f * (c->K / 8), trials + f);
        free(w.app_d);
        free(w.app_p);
        free(w.msg);
        free(w.acc);
        free(w.stamp);
        free(w.touched);
        free(w.pslot);
        free(w.pval);
    }
    return 0;
}

int orc_syndrome_ok(int framesize, int rate, const int16_t* llr)
{
    const orc_code* c = get_code(framesize, rate);
    if (!c)
        return -1;
    int16_t* d = (int16_t*)malloc(c->K * sizeof(int16_t));
    int16_t* p = (int16_t*)malloc(c->R * sizeof(int16_t));
    for (int v = 0; v < c->K; v++)
        d[v] = llr[v];
    for (int idx = 0; idx < c->R; idx++)
        p[M * (idx % c->q) + idx / c->q] = llr[c->K + idx];
    int ok = syndrome_ok(c, d, p);
    free(d);
    free(p);
    return ok;
}

/* ------------------------------------------------------------------------ */
/* IRA encoder (reference ldpc_encode.cc:6-13)                                */
/* ------------------------------------------------------------------------ */

int orc_ldpc_encode(int framesize, int rate, const uint8_t* info, uint8_t* cw, int B)
{
    const orc_code* c = get_code(framesize, rate);
    if (!c)
        return -1;
    const int K = c->K, q = c->q, N = c->N;
    const size_t R = (size_t)c->R;
#ifdef _OPENMP
#pragma omp parallel for
#endif
    for (int f = 0; f < B; f++) {
        const uint8_t* in = info + (size_t)f * (K / 8);
        uint8_t* out = cw + (size_t)f * (N / 8);
        uint8_t* par = (uint8_t*)calloc(R, 1);
        const uint16_t* a = c->src->addr;
        int o = 0;
        for (int r = 0; r < c->src->n_rows; r++) {
            const int d = c->src->row_deg[r];
            for (int jj = 0; jj < M; jj++) {
                const int bit = r * M + jj;
                if ((in[bit >> 3] >> (7 - (bit & 7))) & 1)
                    for (int n = 0; n < d; n++)
                        par[(a[o + n] + (size_t)jj * q) % R] ^= 1;
            }
            o += d;
        }
        for (size_t k = 1; k < R; k++)
            par[k] ^= par[k - 1];
        memcpy(out, in, K / 8);
        memset(out + K / 8, 0, R / 8);
        for (size_t k = 0; k < R; k++)
            if (par[k])
                out[(K + k) >> 3] |= (uint8_t)(1 << (7 - ((K + k) & 7)));
        free(par);
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* BCH (reference fec/bch_code.cc, lib/qa_bch_code.cc:17-32)                 */
/* ------------------------------------------------------------------------ */

int orc_bch_generator(int framesize, int rate, uint64_t gen[4])
{
    const orc_code* c = get_code(framesize, rate);
    if (!c)
        return -1;
    memcpy(gen, c->gen, sizeof(c->gen));
    return c->p;
}

/* r <- (r * x + b * x^p) mod g for one input bit b, r of degree < p. */
static inline void lfsr_step(uint64_t* r, const uint64_t* g, int p, int b)
{
    const int fb = (int)((r[(p - 1) >> 6] >> ((p - 1) & 63)) & 1) ^ b;
    for (int w = 3; w > 0; w--)
        r[w] = (r[w] << 1) | (r[w - 1] >> 63);
    r[0] <<= 1;
    /* keep degree < p */
    for (int w = 0; w < 4; w++) {
        const int lo = 64 * w;
        if (p <= lo)
            r[w] = 0;
        else if (p < lo + 64)
            r[w] &= (1ull << (p - lo)) - 1;
    }
    if (fb)
        for (int w = 0; w < 4; w++)
            r[w] ^= g[w];
    /* g's x^p term fell outside the mask */
    for (int w = 0; w < 4; w++) {
        const int lo = 64 * w;
        if (p <= lo)
            r[w] = 0;
        else if (p < lo + 64)
            r[w] &= (1ull << (p - lo)) - 1;
    }
}

static void remainder_bits(const orc_code* c, const uint8_t* bytes, int nbits, uint64_t* r)
{
    memset(r, 0, 4 * sizeof(uint64_t));
    for (int i = 0; i < nbits; i++)
        lfsr_step(r, c->gen, c->p, (bytes[i >> 3] >> (7 - (i & 7))) & 1);
}

static uint8_t rem_byte(const uint64_t* r, int lo)
{
    uint8_t v = 0;
    for (int b = 0; b < 8; b++)
        if ((r[(lo + b) >> 6] >> ((lo + b) & 63)) & 1)
            v |= (uint8_t)(1 << b);
    return v;
}

int orc_bch_encode(int framesize, int rate, const uint8_t* msg, uint8_t* cw, int B)
{
    const orc_code* c = get_code(framesize, rate);
    if (!c)
        return -1;
    const int kb = c->k_bch / 8, nb = c->n_bch / 8, p = c->p;
#ifdef _OPENMP
#pragma omp parallel for
#endif
    for (int f = 0; f < B; f++) {
        uint64_t r[4];
        remainder_bits(c, msg + (size_t)f * kb, c->k_bch, r);
        memcpy(cw + (size_t)f * nb, msg + (size_t)f * kb, kb);
        for (int j = 0; j < p / 8; j++)
            cw[(size_t)f * nb + kb + j] = rem_byte(r, p - 8 * (j + 1));
    }
    return 0;
}

int orc_bch_check(int framesize, int rate, const uint8_t* cw, uint8_t* rem, int32_t* valid, int B)
{
    const orc_code* c = get_code(framesize, rate);
    if (!c)
        return -1;
    const int nb = c->n_bch / 8, p = c->p;
#ifdef _OPENMP
#pragma omp parallel for
#endif
    for (int f = 0; f < B; f++) {
        uint64_t r[4];
        remainder_bits(c, cw + (size_t)f * nb, c->n_bch, r);
        int any = 0;
        for (int j = 0; j < p / 8; j++) {
            uint8_t b = rem_byte(r, p - 8 * (j + 1));
            if (rem)
                rem[(size_t)f * (p / 8) + j] = b;
            any |= b;
        }
        valid[f] = any == 0;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Demapper (reference cuda/demapper_kernel.cu:31-184)                       */
/* ------------------------------------------------------------------------ */

/* e^-x for 0 <= x < 88: 2^-(x log2 e) = 2^-n * e^(-f ln 2), |f| <= 1/2, with
 * the degree-7 Taylor polynomial of e^u evaluated by Horner in fused
 * multiply-adds. */
float orc_exp_neg(float x)
{
    const float t = x * 1.44269504088896341f;
    const float n = rintf(t);
    const float f = t - n;
    const float u = -(f * 0.693147180559945309f);
    float p = 1.98412698412698413e-4f;          /* 1/7! */
    p = fmaf(p, u, 1.38888888888888889e-3f);     /* 1/6! */
    p = fmaf(p, u, 8.33333333333333333e-3f);     /* 1/5! */
    p = fmaf(p, u, 4.16666666666666667e-2f);     /* 1/4! */
    p = fmaf(p, u, 1.66666666666666667e-1f);     /* 1/3! */
    p = fmaf(p, u, 0.5f);
    p = fmaf(p, u, 1.0f);
    p = fmaf(p, u, 1.0f);
    const int ni = (int)n;
    union { uint32_t u; float f; } sc;
    sc.u = (uint32_t)(127 - ni) << 23;
    return p * sc.f;
}

/* ln x for normal x > 0: x = m 2^e, m in [sqrt(1/2), sqrt 2),
 * ln m = 2 atanh(s), s = (m-1)/(m+1), series to s^9. */
float orc_log(float x)
{
    union { uint32_t u; float f; } b;
    b.f = x;
    int e = (int)((b.u >> 23) & 0xff) - 127;
    b.u = (b.u & 0x7fffffu) | 0x3f800000u;
    float m = b.f;
    if (m > 1.41421356237309505f) {
        m = m * 0.5f;
        e += 1;
    }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    float p = 0.111111111111111111f;             /* 1/9 */
    p = fmaf(p, s2, 0.142857142857142857f);      /* 1/7 */
    p = fmaf(p, s2, 0.2f);
    p = fmaf(p, s2, 0.333333333333333333f);
    p = fmaf(p, s2, 1.0f);
    const float l = (2.0f * s) * p;
    return fmaf((float)e, 0.693147180559945309f, l);
}

static inline int16_t llr_round(float v)
{
    v = rintf(v);
    v = fminf(fmaxf(v, -32768.0f), 32767.0f);
    return (int16_t)v;
}

/* Loudest-bit squared distance (demapper_kernel.cu:216-237).  The float
 * sums are evaluated without contraction (the oracle is built with
 * -ffp-contract=off), like the reference's host code. */
float orc_demap_dmax(int kind, const float* pts_re, const float* pts_im, int n_points, int n_mod)
{
    if (kind == 0)
        return 2.0f;
    if (kind == 1)
        return 4.0f;
    float dmax = 0.0f;
    for (int i = 0; i < n_points; i++) {
        for (int b = 0; b < n_mod; b++) {
            const int mask = 1 << (n_mod - 1 - b);
            float dmin = 1e30f;
            for (int k = 0; k < n_points; k++) {
                if (((i ^ k) & mask) == 0)
                    continue;
                const float dr = pts_re[i] - pts_re[k];
                const float di = pts_im[i] - pts_im[k];
                const float d = dr * dr + di * di;
                if (d < dmin)
                    dmin = d;
            }
            if (dmin > dmax)
                dmax = dmin;
        }
    }
    return dmax;
}

/* demapper_cuda::capped_llr_gain (demapper_kernel.cu:283-291) */
float orc_capped_llr_gain(float dmax, float llr_target, float llr_gain)
{
    if (llr_target <= 0.0f || dmax <= 0.0f)
        return llr_gain;
    const float cap = 2.0f * llr_target / dmax;
    return llr_gain < cap ? llr_gain : cap;
}

int orc_demap(const float* sym, int B, int xfec, int interleaved_len, int fec_len, int n_mod,
              int kind, const float* pts_re, const float* pts_im, int n_points,
              const uint32_t* col, float noise_var, float llr_gain, int16_t* out)
{
#ifdef _OPENMP
#pragma omp parallel for
#endif
    for (int cw = 0; cw < B; cw++) {
        int16_t* o = out + (size_t)cw * fec_len;
        for (int j = 0; j < interleaved_len; j++) {
            const float re = sym[((size_t)cw * xfec + j) * 2];
            const float im = sym[((size_t)cw * xfec + j) * 2 + 1];
            if (kind == 0) {
                const float scalar = (2.0f * 1.4142135623730951f) / noise_var;
                const int pos = 2 * j;
                if (pos + 1 < fec_len) {
                    o[pos] = llr_round(re * scalar);
                    o[pos + 1] = llr_round(im * scalar);
                }
            } else if (kind == 1) {
                const float C8 = 0.92387953251128676f, S8 = 0.38268343236508977f;
                const float R2 = 0.70710678118654752f;
                const float DIST = 2.0f * 0.38268343236508977f;
                const float cr = fmaf(re, C8, im * S8);
                const float ci = fmaf(-re, S8, im * C8);
                const float scale = DIST * llr_gain;
                const float l0 = (R2 * (fabsf(cr) - fabsf(ci))) * scale;
                const float l1 = cr * scale;
                const float l2 = ci * scale;
                o[col[0] + j] = llr_round(l0);
                o[col[1] + j] = llr_round(l1);
                o[col[2] + j] = llr_round(l2);
            } else {
                float min0[8], min1[8], s0[8], s1[8];
                for (int b = 0; b < 8; b++) {
                    min0[b] = 1e30f;
                    min1[b] = 1e30f;
                    s0[b] = 0.0f;
                    s1[b] = 0.0f;
                }
                for (int i = 0; i < n_points; i++) {
                    const float dr = re - pts_re[i], di = im - pts_im[i];
                    const float d = fmaf(dr, dr, di * di);
                    for (int b = 0; b < n_mod; b++) {
                        if (i & (1 << (n_mod - 1 - b))) {
                            if (d < min1[b])
                                min1[b] = d;
                        } else {
                            if (d < min0[b])
                                min0[b] = d;
                        }
                    }
                }
                const float scale = llr_gain * 0.25f;
                for (int i = 0; i < n_points; i++) {
                    const float dr = re - pts_re[i], di = im - pts_im[i];
                    const float d = fmaf(dr, dr, di * di);
                    for (int b = 0; b < n_mod; b++) {
                        if (i & (1 << (n_mod - 1 - b))) {
                            const float delta = (d - min1[b]) * scale;
                            if (delta < 16.0f)
                                s1[b] = s1[b] + orc_exp_neg(delta);
                        } else {
                            const float delta = (d - min0[b]) * scale;
                            if (delta < 16.0f)
                                s0[b] = s0[b] + orc_exp_neg(delta);
                        }
                    }
                }
                for (int b = 0; b < n_mod; b++) {
                    const float corr = 2.0f * (orc_log(fmaxf(s0[b], 1e-30f)) - orc_log(fmaxf(s1[b], 1e-30f)));
                    const float llr = fmaf(min1[b] - min0[b], llr_gain * 0.5f, corr);
                    const uint32_t pos = col[b] + (uint32_t)j;
                    if (pos < (uint32_t)fec_len)
                        o[pos] = llr_round(llr);
                }
            }
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Mapper (reference cuda/mapper_kernel.cu:22-51, mapper.cc:75-86)           */
/* ------------------------------------------------------------------------ */

int orc_map(const uint8_t* cw, int B, int cw_bytes, int xfec, int interleaved_len, int fec_len, int n_mod,
            const uint32_t* col, int stride, const float* pts_re, const float* pts_im, float* sym)
{
    for (int f = 0; f < B; f++) {
        const uint8_t* in = cw + (size_t)f * cw_bytes;
        for (int j = 0; j < xfec; j++) {
            int label = (1 << n_mod) - 1;
            if (j < interleaved_len) {
                label = 0;
                for (int b = 0; b < n_mod; b++) {
                    const int pos = (int)col[b] + j * stride;
                    const int bit = pos < fec_len ? (in[pos >> 3] >> (7 - (pos & 7))) & 1 : 0;
                    label |= bit << (n_mod - 1 - b);
                }
            }
            sym[((size_t)f * xfec + j) * 2] = pts_re[label];
            sym[((size_t)f * xfec + j) * 2 + 1] = pts_im[label];
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Unrolled learned min-sum (training model), float and double copies       */
/* ------------------------------------------------------------------------ */

/* Largest number of edges of a check (two parity edges + circulants). */
static int nms_edge_width(const orc_code* c)
{
    int w = 0;
    for (int i = 0; i < c->q; i++)
        if (c->lay_off[i + 1] - c->lay_off[i] + 2 > w)
            w = c->lay_off[i + 1] - c->lay_off[i] + 2;
    return w;
}

#define REAL float
#define SFX(n) n##_f32
#include "nms_model.inc"
#undef REAL
#undef SFX
#define REAL double
#define SFX(n) n##_f64
#include "nms_model.inc"
#undef REAL
#undef SFX

/* ------------------------------------------------------------------------ */
/* Post-FEC baseband stage                                                  */
/* ------------------------------------------------------------------------ */

/* BB scrambler PRBS (EN 302 307-1 clause 5.2.2, figure 5; reference
 * bb_scrambler.cc:18-40): 1 + X^14 + X^15, register loaded with
 * 100101010000000 (stage 1 first) at the start of every BBFRAME, output bits
 * MSB first. */
void orc_bb_prbs(uint8_t* seq, int n_bytes)
{
    const char* init = "100101010000000";
    unsigned reg = 0;
    for (int s = 0; s < 15; s++)
        if (init[s] == '1')
            reg |= 1u << s;
    for (int i = 0; i < n_bytes; i++) {
        uint8_t byte = 0;
        for (int b = 0; b < 8; b++) {
            const unsigned out = ((reg >> 13) ^ (reg >> 14)) & 1u;
            reg = ((reg << 1) | out) & 0x7fffu;
            byte = (uint8_t)((byte << 1) | out);
        }
        seq[i] = byte;
    }
}

/* CRC-8 of the BBHEADER (x^8 + x^7 + x^6 + x^4 + x^2 + 1, register cleared,
 * MSB first; reference fec/crc8.h). */
static uint8_t crc8_bb(const uint8_t* d, int n)
{
    uint8_t reg = 0;
    for (int i = 0; i < n; i++) {
        reg ^= d[i];
        for (int b = 0; b < 8; b++)
            reg = (reg & 0x80) ? (uint8_t)((reg << 1) ^ 0xD5) : (uint8_t)(reg << 1);
    }
    return reg;
}

/* The RX chain's post-FEC loop (reference rx_fec_chain.cc:604-626 with
 * bbframe_parser.cc:14-56): a frame is used only if its LDPC decode
 * converged and its BCH check passed; it is descrambled, its BBHEADER must
 * have a zero CRC over its 10 bytes, DFL <= 8 kbch - 80, DFL % 8 == 0 and
 * TS/GS = generic packetized; then its DFL/8 data-field bytes are appended
 * to out if they fit in the room left (else the frame yields nothing).
 * lengths[f] = bytes appended for frame f, offsets[f] = where; offsets[B] =
 * total. */
int orc_bb_extract(const uint8_t* hard, int stride, int kbch, const int32_t* trials, const int32_t* valid, int B,
                   uint8_t* out, int max_out, int32_t* lengths, int32_t* offsets)
{
    if (kbch < 10 || kbch > 7274)
        return -1;
    uint8_t* prbs = (uint8_t*)malloc((size_t)kbch);
    uint8_t* fr = (uint8_t*)malloc((size_t)kbch);
    if (!prbs || !fr) {
        free(prbs);
        free(fr);
        return -2;
    }
    orc_bb_prbs(prbs, kbch);
    int used = 0;
    for (int f = 0; f < B; f++) {
        int n = 0;
        offsets[f] = used;
        if (trials[f] >= 0 && valid[f]) {
            for (int i = 0; i < kbch; i++)
                fr[i] = (uint8_t)(hard[(size_t)f * stride + i] ^ prbs[i]);
            const int dfl = (fr[4] << 8) | fr[5];
            const int ts_gs = fr[0] >> 6;
            if (crc8_bb(fr, 10) == 0 && dfl <= 8 * kbch - 80 && dfl % 8 == 0 && ts_gs == 0) {
                n = dfl / 8;
                if (n > max_out - used)
                    n = 0;
                else
                    memcpy(out + used, fr + 10, (size_t)n);
            }
        }
        lengths[f] = n;
        used += n;
    }
    offsets[B] = used;
    free(prbs);
    free(fr);
    return 0;
}

/* A scrambled GSE BBFRAME of kbch bytes carrying data[0..len) (test traffic;
 * the header layout of reference bb_header.cc:28-49: MATYPE-1 with TS/GS =
 * matype_ts_gs, SIS = 1, CCM, roll-off 0.20; UPL = 0; DFL = 8 len; SYNC = 0;
 * SYNCD = 0xFFFF; CRC-8), zero padding, then the PRBS. */
int orc_bb_build(const uint8_t* data, int len, int kbch, int matype_ts_gs, uint8_t* out)
{
    if (len < 0 || len > kbch - 10)
        return -1;
    memset(out, 0, (size_t)kbch);
    out[0] = (uint8_t)(((matype_ts_gs & 3) << 6) | 0x20 | 0x10 | 0x02);
    out[4] = (uint8_t)((8 * len) >> 8);
    out[5] = (uint8_t)(8 * len);
    out[7] = 0xFF;
    out[8] = 0xFF;
    out[9] = crc8_bb(out, 9);
    memcpy(out + 10, data, (size_t)len);
    uint8_t* prbs = (uint8_t*)malloc((size_t)kbch);
    if (!prbs)
        return -2;
    orc_bb_prbs(prbs, kbch);
    for (int i = 0; i < kbch; i++)
        out[i] ^= prbs[i];
    free(prbs);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Decision-directed SNR estimate (reference modulation/dd_snr.cc:12-47 and  */
/* nearest_label, modulation/constellation.cc:495-507)                       */
/* ------------------------------------------------------------------------ */

float orc_dd_snr(const float* sym, int n_sym, const float* pts, int n_points, int stride, int qpsk)
{
    float sig = 0.0f, err = 0.0f;
    if (qpsk) {
        const float h = 0.70710678f;
        for (int i = 0; i < n_sym; i++) {
            float x = sym[2 * i], y = sym[2 * i + 1];
            float a = x < 0 ? -h : h, b = y < 0 ? -h : h;
            float ex = x - a, ey = y - b;
            sig += a * a + b * b;
            err += ex * ex;
            err += ey * ey;
        }
    } else {
        for (int i = 0; i < n_sym; i += stride) {
            float x = sym[2 * i], y = sym[2 * i + 1];
            int k = 0;
            float dk = FLT_MAX;
            for (int l = 0; l < n_points; l++) {
                float u = x - pts[2 * l], v = y - pts[2 * l + 1];
                float d = u * u + v * v;
                if (d < dk) {
                    dk = d;
                    k = l;
                }
            }
            float px = pts[2 * k], py = pts[2 * k + 1];
            float ex = x - px, ey = y - py;
            sig += px * px + py * py;
            err += ex * ex + ey * ey;
        }
    }
    if (!isfinite(sig) || !isfinite(err))
        return 0.0f;
    return err * 1e6f <= sig ? 1e6f : sig / err;
}

/* ------------------------------------------------------------------------ */
/* PL receiver tail: descrambling and pilot removal                          */
/* ------------------------------------------------------------------------ */

/* Rotation index R_n(i) of the PLFRAME scrambler (EN 302 307-1 clause
 * 5.5.4; reference framing/pl_scrambler.cc:47-71): the m-sequences
 * x(i + 18) = x(i + 7) + x(i), x(0) = 1, x(1..17) = 0, and
 * y(i + 18) = y(i + 10) + y(i + 7) + y(i + 5) + y(i), y(0..17) = 1 (mod 2),
 * period P = 2^18 - 1, are written out in full; z_n(i) = x(i + n) + y(i) and
 * R_n(i) = 2 z_n(i + 2^17) + z_n(i), indices mod P.  The descrambling
 * factor is e^{-j R pi/2}.  Returns -1 for n outside 0 .. 2^18 - 3. */
#define PL_PERIOD 262143
int orc_pl_rotation(int gold, uint8_t* r, int len)
{
    if (gold < 0 || gold >= PL_PERIOD - 1 || len < 0)
        return -1;
    uint8_t* x = (uint8_t*)malloc(PL_PERIOD + 18);
    uint8_t* y = (uint8_t*)malloc(PL_PERIOD + 18);
    memset(x, 0, 18);
    x[0] = 1;
    memset(y, 1, 18);
    for (int i = 0; i + 18 < PL_PERIOD + 18; i++) {
        x[i + 18] = x[i + 7] ^ x[i];
        y[i + 18] = y[i + 10] ^ y[i + 7] ^ y[i + 5] ^ y[i];
    }
    for (int i = 0; i < len; i++) {
        const int i0 = i % PL_PERIOD, i1 = (i + 131072) % PL_PERIOD;
        const int z0 = x[(i0 + gold) % PL_PERIOD] ^ y[i0];
        const int z1 = x[(i1 + gold) % PL_PERIOD] ^ y[i1];
        r[i] = (uint8_t)(2 * z1 + z0);
    }
    free(x);
    free(y);
    return 0;
}

/* The data symbols of one located PLFRAME (reference plrx/pl_receiver.cc
 * :1694-1741 with rotate_slot :1217-1282): payload = the symbols after the
 * 90-symbol PLHEADER; slot s (90 symbols) starts at s * 90 + min(s / 16,
 * pilot blocks) * 36 (a 36-symbol pilot block after every 16 slots,
 * (slots - 1) / 16 blocks when pilots are on); each symbol is descrambled
 * (times e^{-j R pi/2}) and counter-rotated: symbol i of the slot is
 * multiplied by rot * step^i, with the powers built as four interleaved
 * chains (chain c = i mod 4 starts at rot * step^c and advances by step^4),
 * every product in the reference's order, no contraction; non-finite
 * results become 0.  slot_rot: per slot {rot re, rot im, step re, step im},
 * or NULL for rot = step = 1.  out: 90 * slots (re, im) pairs. */
int orc_pl_extract(const float* payload, int slots, int pilots, const uint8_t* r, const float* slot_rot, float* out)
{
    static const float ROT_RE[4] = {1.0f, 0.0f, -1.0f, 0.0f};
    static const float ROT_IM[4] = {0.0f, -1.0f, 0.0f, 1.0f};
    if (slots <= 0 || !payload || !r || !out)
        return -1;
    const int n_pb = pilots ? (slots - 1) / 16 : 0;
    for (int s = 0; s < slots; s++) {
        const int off = s * 90 + (s / 16 < n_pb ? s / 16 : n_pb) * 36;
        const float rr = slot_rot ? slot_rot[4 * s] : 1.0f, ri = slot_rot ? slot_rot[4 * s + 1] : 0.0f;
        const float sr = slot_rot ? slot_rot[4 * s + 2] : 1.0f, si = slot_rot ? slot_rot[4 * s + 3] : 0.0f;
        float cr[4], ci[4];
        cr[0] = rr;
        ci[0] = ri;
        for (int c = 1; c < 4; c++) {
            cr[c] = cr[c - 1] * sr - ci[c - 1] * si;
            ci[c] = cr[c - 1] * si + ci[c - 1] * sr;
        }
        float pr = sr, pi = si;
        for (int c = 1; c < 4; c++) {
            const float t = pr * sr - pi * si;
            pi = pr * si + pi * sr;
            pr = t;
        }
        float* o = out + 2 * (size_t)s * 90;
        for (int i = 0; i < 90; i++) {
            const int c = i & 3, k = off + i;
            const float ar = payload[2 * k], ai = payload[2 * k + 1];
            const float br = ROT_RE[r[k] & 3], bi = ROT_IM[r[k] & 3];
            const float xr = ar * br - ai * bi, xi = ar * bi + ai * br;
            float vr = xr * cr[c] - xi * ci[c], vi = xr * ci[c] + xi * cr[c];
            if (i < 88) {  /* the chains advance once per group of four */
                const float nr = cr[c] * pr - ci[c] * pi;
                ci[c] = cr[c] * pi + ci[c] * pr;
                cr[c] = nr;
            }
            if (!isfinite(vr) || !isfinite(vi))
                vr = vi = 0.0f;
            o[2 * i] = vr;
            o[2 * i + 1] = vi;
        }
    }
    return 0;
}
