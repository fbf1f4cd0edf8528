// Decoding plans of the DVB-S2/S2X LDPC codes, BCH tables, and the
// product-side encoders.
//
// Plan layout.  Check j of layer i is parity check p = q*j + i (the
// reference's transposed order, lib/cusat_dsp/cuda/ldpc_decode_kernel.cu:
// 1021-1031).  Information bit g*360 + m with accumulator address x checks
// (x + m q) mod R, so it lies in layer x mod q at check j = (x div q + m)
// mod 360: each address of a table row is one circulant of one layer, and
// check j of the layer reads bit g*360 + (j - x div q) mod 360.  The plan
// stores one descriptor word per (layer, circulant) instead of the
// reference's per-edge position table (R * CNL u16, .cu:1006-1031).
#include <mutex>
#include <stdexcept>
#include <string.h>

#include "host.h"

extern "C" {
#include "cusat_data.h"
#include "gen/code_tables.inc"
}

#include "fec_consts.h"

namespace cusat {

int cmax_bucket(int cnt_max)
{
    // one kernel instantiation per bucket: with packed pairs of edges a
    // check row of cmax + 2 slots wastes at most one half (an absent slot
    // or the pad), the common DVB-S2 codes fit exactly
    static const int buckets[] = {2, 3, 4, 5, 6, 8, 9, 10, 12, 14, 16, 18, 20, 26, 28};
    for (int b : buckets)
        if (cnt_max <= b)
            return b;
    return -1;
}

namespace {

int poly_degree(const uint64_t* a)
{
    for (int i = 255; i >= 0; i--)
        if ((a[i >> 6] >> (i & 63)) & 1)
            return i;
    return -1;
}

// Builds the plan; throws std::runtime_error with a message on failure.
void build_plan(CodePlan& c, int framesize, int rate)
{
    const char* name = cusat_table_name(framesize, rate);
    const cusat_bch_row* br = cusat_find_bch_row(framesize, rate);
    if (!name || !br)
        throw std::runtime_error("no LDPC/BCH code for this frame size and rate");
    const cusat_table_src* src = nullptr;
    for (int i = 0; i < CUSAT_N_TABLE_SRCS; i++)
        if (!strcmp(cusat_table_srcs[i].name, name))
            src = &cusat_table_srcs[i];
    if (!src)
        throw std::runtime_error("parity-check table missing");
    c.framesize = framesize;
    c.rate = rate;
    c.name = name;
    c.N = src->n;
    c.K = src->k;
    c.R = c.N - c.K;
    c.q = c.R / kM;
    c.links_total = src->links_total;
    c.row_deg = src->row_deg;
    c.addr = src->addr;
    c.n_rows = src->n_rows;
    const int q = c.q;

    // circulants per layer, in table order
    std::vector<std::vector<std::pair<int, int>>> lay(q);  // (group, shift)
    c.dv_max = 0;
    for (int r = 0, o = 0; r < src->n_rows; r++) {
        c.dv_max = std::max(c.dv_max, (int)src->row_deg[r]);
        for (int d = 0; d < src->row_deg[r]; d++, o++)
            lay[src->addr[o] % q].push_back({r, src->addr[o] / q});
    }
    c.cnt_max = 0;
    c.cnt.resize(q);
    for (int i = 0; i < q; i++) {
        c.cnt[i] = (uint8_t)lay[i].size();
        c.cnt_max = std::max(c.cnt_max, (int)lay[i].size());
        if (lay[i].empty())
            throw std::runtime_error("layer without information circulants");
    }
    c.cmax = cmax_bucket(c.cnt_max);
    if (c.cmax < 0)
        throw std::runtime_error("check degree above the largest kernel bucket");
    // no information bit of the frame may push |APP| past int16 when every
    // channel LLR is within fast_lim: |APP| <= |llr| + 127 * (deg + 1)
    c.fast_lim = 32767 - 127 * (c.dv_max + 2);

    // schedule: the paired schedule built for this table when its layer
    // count matches, else one layer per step (reference
    // ldpc_decode_kernel.cu:1118-1170, ldpc_schedule_registry.h:102-106)
    const cusat_sched_src* ss = nullptr;
    for (int i = 0; i < CUSAT_N_SCHED_SRCS; i++)
        if (!strcmp(cusat_sched_srcs[i].name, name) && cusat_sched_srcs[i].q == q)
            ss = &cusat_sched_srcs[i];
    if (ss) {
        c.n_steps = ss->n_steps;
        c.sched.assign(ss->pairs, ss->pairs + 2 * ss->n_steps);
        c.lanes = 2;
    } else {
        c.n_steps = q;
        c.sched.resize(2 * q);
        for (int i = 0; i < q; i++) {
            c.sched[2 * i] = (int16_t)i;
            c.sched[2 * i + 1] = -1;
        }
        c.lanes = 1;
    }
    c.msg_row = 4 * row_words(c.cmax, c.lanes);

    // Shared groups per step: a group (table row) reached by several
    // circulants of one step has its bits updated by all of them.  Each such
    // circulant gets its own stage row (rows of one group consecutive, sets
    // alternating with the step parity); a group item completes the bits.
    // Every layer occurs in exactly one step, so a slot's staging is a
    // property of the plan.
    std::vector<std::vector<int>> srow(q);   // stage row per circulant, -1 = plain
    std::vector<std::vector<int>> sset(q);
    for (int i = 0; i < q; i++) {
        srow[i].assign(lay[i].size(), -1);
        sset[i].assign(lay[i].size(), 0);
    }
    c.step_conf.assign(c.n_steps, 0);
    c.item_off.assign(c.n_steps + 1, 0);
    c.items.clear();
    c.max_stage = 0;
    std::vector<std::vector<int>> shared_groups(c.n_steps);
    std::vector<std::vector<int>> step_groups(c.n_steps);
    for (int s = 0; s < c.n_steps; s++) {
        struct Ref { int layer, slot, group; };
        std::vector<Ref> refs;
        for (int l = 0; l < 2; l++) {
            const int i = c.sched[2 * s + l];
            if (i >= 0)
                for (int e = 0; e < (int)lay[i].size(); e++) {
                    refs.push_back({i, e, lay[i][e].first});
                    step_groups[s].push_back(lay[i][e].first);
                }
        }
        std::vector<int> mult(src->n_rows, 0), first_row(src->n_rows, -1), used(src->n_rows, 0);
        for (auto& r : refs)
            mult[r.group]++;
        int next_row = 0;
        for (auto& r : refs) {
            if (mult[r.group] < 2)
                continue;
            if (first_row[r.group] < 0) {
                first_row[r.group] = next_row;
                next_row += mult[r.group];
                shared_groups[s].push_back(r.group);
                c.items.push_back((uint32_t)(2 * r.group * kM));
                c.items.push_back((uint32_t)first_row[r.group] | ((uint32_t)mult[r.group] << 8));
            }
            srow[r.layer][r.slot] = first_row[r.group] + used[r.group]++;
            sset[r.layer][r.slot] = s & 1;
        }
        if (next_row > kMaxStage)
            throw std::runtime_error("step needs more stage rows than the kernel has");
        c.max_stage = std::max(c.max_stage, next_row);
        c.item_off[s + 1] = (uint16_t)(c.items.size() / 2);
    }
    // completion of a step's shared groups: deferred into the next step when
    // that step does not touch them, else after a barrier inside the step
    for (int s = 0; s < c.n_steps; s++) {
        if (shared_groups[s].empty())
            continue;
        bool defer = s + 1 < c.n_steps;
        if (defer)
            for (int g : shared_groups[s])
                for (int g2 : step_groups[s + 1])
                    if (g == g2)
                        defer = false;
        c.step_conf[s] = defer ? kConfDefer : kConfMid;
    }
    // slot descriptors
    c.tab.assign((size_t)q * c.cmax * 4, 0);
    for (int i = 0; i < q; i++)
        for (int e = 0; e < c.cmax; e++) {
            uint32_t* t = &c.tab[((size_t)i * c.cmax + e) * 4];
            if (e >= (int)lay[i].size()) {
                t[0] = 0;
                t[1] = 0;
                t[2] = (uint32_t)(2 * kM);  // junk region follows the dummy region
                t[3] = kSlotAbsent;
                continue;
            }
            const int g = lay[i][e].first, sh = lay[i][e].second;
            t[0] = (uint32_t)(2 * g * kM);
            t[1] = (uint32_t)((kM - sh) % kM);
            if (srow[i][e] < 0) {
                t[2] = 0;
                t[3] = kSlotPlain;
            } else {
                // stage entry (relative to the stage region) minus the APP slot
                const int rel = (sset[i][e] * kMaxStage + srow[i][e]) * 2 * kM;
                t[2] = (uint32_t)(rel - 2 * g * kM);
                t[3] = kSlotStaged;
            }
        }

    // BCH outer code: g = g1 g2 ... gt (reference fec/bch_code.cc:99-122)
    c.k_bch = (int)br->k_bch;
    c.n_bch = (int)br->n_bch;
    c.t = (int)br->t;
    memset(c.gen, 0, sizeof(c.gen));
    c.gen[0] = 1;
    const int fam = framesize == CUSAT_FECFRAME_NORMAL ? 0 : framesize == CUSAT_FECFRAME_SHORT ? 1 : 2;
    for (int i = 0; i < c.t; i++) {
        uint64_t r[4] = {0, 0, 0, 0};
        const uint32_t b = cusat_bch_minpoly[fam][i];
        for (int sh = 0; sh < 32; sh++) {
            if (!((b >> sh) & 1))
                continue;
            for (int w = 3; w >= 0; w--) {
                uint64_t v = c.gen[w] << sh;
                if (sh && w > 0)
                    v |= c.gen[w - 1] >> (64 - sh);
                r[w] ^= v;
            }
        }
        memcpy(c.gen, r, sizeof(r));
    }
    c.p = poly_degree(c.gen);
    if (c.n_bch != c.K || c.k_bch != c.n_bch - c.p)
        throw std::runtime_error("inconsistent BCH/LDPC dimensions");
}

}  // namespace

const CodePlan* get_code_plan(int framesize, int rate, std::string* err)
{
    static std::mutex mu;
    static std::vector<CodePlan*> cache(3 * CUSAT_RATE_COUNT, nullptr);
    static std::vector<std::string> errors(3 * CUSAT_RATE_COUNT);
    static std::vector<char> done(3 * CUSAT_RATE_COUNT, 0);
    if (framesize < 0 || framesize > 2 || rate < 0 || rate >= CUSAT_RATE_COUNT) {
        if (err)
            *err = "frame size or rate out of range";
        return nullptr;
    }
    const int k = framesize * CUSAT_RATE_COUNT + rate;
    std::lock_guard<std::mutex> lock(mu);
    if (!done[k]) {
        done[k] = 1;
        CodePlan* c = new CodePlan();
        try {
            build_plan(*c, framesize, rate);
            cache[k] = c;
        } catch (const std::exception& e) {
            errors[k] = e.what();
            delete c;
        }
    }
    if (!cache[k] && err)
        *err = errors[k];
    return cache[k];
}

// ---------------------------------------------------------------------------
// BCH tables
// ---------------------------------------------------------------------------

namespace {

// x^e mod g for e = 0..emax, W words each.
std::vector<uint64_t> powers_mod(const uint64_t* gen, int p, size_t emax, int W)
{
    std::vector<uint64_t> pw((emax + 1) * W, 0);
    pw[0] = 1;
    const uint64_t top_mask = (p % 64) ? ((1ull << (p % 64)) - 1) : ~0ull;
    for (size_t e = 1; e <= emax; e++) {
        const uint64_t* a = &pw[(e - 1) * W];
        uint64_t* b = &pw[e * W];
        const int carry = (int)((a[(p - 1) / 64] >> ((p - 1) % 64)) & 1);
        for (int w = W - 1; w >= 0; w--)
            b[w] = (a[w] << 1) | (w ? a[w - 1] >> 63 : 0);
        b[W - 1] &= top_mask;
        if (carry)
            for (int w = 0; w < W; w++)
                b[w] ^= gen[w];
        b[W - 1] &= top_mask;
    }
    return pw;
}

}  // namespace

void bch_encoder_lut(const uint64_t* gen, int p, uint64_t* lut)
{
    const int W = 4;
    std::vector<uint64_t> pw = powers_mod(gen, p, p + 8, W);
    for (int b = 0; b < 256; b++) {
        uint64_t acc[4] = {0, 0, 0, 0};
        for (int bit = 0; bit < 8; bit++)
            if ((b >> bit) & 1)
                for (int w = 0; w < W; w++)
                    acc[w] ^= pw[(size_t)(p + bit) * W + w];
        for (int w = 0; w < W; w++)
            lut[b * 4 + w] = acc[w];
    }
}

bool build_bch_tables(const uint64_t* gen, int p, unsigned n_bytes, BchTables* t, std::string* err)
{
    if (p < 8 || p > 248 || (p & 7) || !(gen[0] & 1) || !((gen[p / 64] >> (p % 64)) & 1) ||
        n_bytes <= (unsigned)(p / 8)) {
        if (err)
            *err = "invalid BCH generator or geometry";
        return false;
    }
    const int W = (p + 63) / 64;
    t->p = p;
    t->words = W;
    t->bytes = p / 8;
    t->n_bytes = n_bytes;
    t->chunk = (n_bytes + 31) / 32;
    t->lead = 32 * t->chunk - n_bytes;
    const size_t emax = (size_t)8 * t->chunk * 16 + p + 8;
    std::vector<uint64_t> pw = powers_mod(gen, p, emax, W);
    t->lut.assign((size_t)256 * W, 0);
    for (int b = 0; b < 256; b++)
        for (int bit = 0; bit < 8; bit++)
            if ((b >> bit) & 1)
                for (int w = 0; w < W; w++)
                    t->lut[(size_t)b * W + w] ^= pw[(size_t)(p + bit) * W + w];
    t->tree.assign((size_t)5 * t->bytes * 256 * W, 0);
    for (int k = 0; k < 5; k++) {
        const size_t shift = (size_t)8 * t->chunk * ((size_t)1 << k);
        for (int j = 0; j < t->bytes; j++)
            for (int b = 1; b < 256; b++) {
                uint64_t* dst = &t->tree[(((size_t)k * t->bytes + j) * 256 + b) * W];
                for (int bit = 0; bit < 8; bit++)
                    if ((b >> bit) & 1)
                        for (int w = 0; w < W; w++)
                            dst[w] ^= pw[(shift + 8 * j + bit) * W + w];
            }
    }
    return true;
}

// ---------------------------------------------------------------------------
// Encoders for generated traffic
// ---------------------------------------------------------------------------

void bch_encode_frames(const CodePlan& c, const uint8_t* msg, uint8_t* cw, int B)
{
    uint64_t lut[256 * 4];
    bch_encoder_lut(c.gen, c.p, lut);
    const int kb = c.k_bch / 8, nb = c.n_bch / 8, p = c.p, pb = p / 8;
    const uint64_t top_mask = (p % 64) ? ((1ull << (p % 64)) - 1) : ~0ull;
    const int W = (p + 63) / 64;
    for (int f = 0; f < B; f++) {
        const uint8_t* in = msg + (size_t)f * kb;
        uint8_t* out = cw + (size_t)f * nb;
        uint64_t r[4] = {0, 0, 0, 0};
        for (int i = 0; i < kb; i++) {
            const int lo = p - 8;
            const unsigned top = (unsigned)((r[lo / 64] >> (lo % 64)) |
                                            ((lo % 64) > 56 && lo / 64 + 1 < 4 ? r[lo / 64 + 1] << (64 - lo % 64) : 0)) & 255u;
            const unsigned idx = top ^ in[i];
            for (int w = W - 1; w >= 0; w--)
                r[w] = (r[w] << 8) | (w ? r[w - 1] >> 56 : 0);
            r[W - 1] &= top_mask;
            for (int w = 0; w < W; w++)
                r[w] ^= lut[idx * 4 + w];
        }
        memcpy(out, in, kb);
        for (int j = 0; j < pb; j++) {
            const int lo = p - 8 * (j + 1);
            uint64_t v = r[lo / 64] >> (lo % 64);
            if ((lo % 64) > 56 && lo / 64 + 1 < 4)
                v |= r[lo / 64 + 1] << (64 - lo % 64);
            out[kb + j] = (uint8_t)v;
        }
    }
}

void ldpc_encode_frames(const CodePlan& c, const uint8_t* info, uint8_t* cw, int B)
{
    const int K = c.K, R = c.R, q = c.q, N = c.N;
    std::vector<uint8_t> par(R);
    for (int f = 0; f < B; f++) {
        const uint8_t* in = info + (size_t)f * (K / 8);
        uint8_t* out = cw + (size_t)f * (N / 8);
        std::fill(par.begin(), par.end(), 0);
        for (int r = 0, o = 0; r < c.n_rows; r++) {
            const int d = c.row_deg[r];
            for (int m = 0; m < kM; m++) {
                const int bit = r * kM + m;
                if (!((in[bit >> 3] >> (7 - (bit & 7))) & 1))
                    continue;
                for (int n = 0; n < d; n++) {
                    int a = c.addr[o + n] + m * q;
                    if (a >= R)
                        a -= R;
                    par[a] ^= 1;
                }
            }
            o += d;
        }
        memcpy(out, in, K / 8);
        uint8_t acc = 0;
        for (int k = 0; k < R; k += 8) {
            uint8_t byte = 0;
            for (int b = 0; b < 8; b++) {
                acc ^= par[k + b];
                byte |= (uint8_t)(acc << (7 - b));
            }
            out[(K + k) / 8] = byte;
        }
    }
}

}  // namespace cusat
