// PL receiver tail on the GPU: located PLFRAMEs -> XFECFRAMEs.
//
// The reference's PL receiver (lib/cusat_dsp/plrx/pl_receiver.cc) finds
// PLHEADERs, decodes the PLS code and tracks carrier phase and amplitude
// with sequential filters; then, per delivered frame, it descrambles the
// payload, drops the pilot blocks and counter-rotates each 90-symbol slot
// (:1694-1741, rotate_slot :1217-1282).  The synchroniser stays on the
// host; this file is that last, data-parallel step for a batch of frames:
// each frame brings its payload (the symbols after the 90-symbol PLHEADER),
// its PLS code (layout: slots, pilot blocks; EN 302 307-1 clause 5.5,
// EN 302 307-2 Tables 17a/17b), its scrambling code and optionally a
// rotation per slot (the phase/gain estimates of the synchroniser), and
// receives its 90 S data symbols -- the XFECFRAME the demapper reads.
//
// Arithmetic follows the reference exactly: the descrambling factor
// e^{-j R pi/2} (R from the Gold sequence, EN 302 307-1 clause 5.5.4) is
// applied as a complex product, symbol i of a slot is multiplied by
// rot * step^i where the powers are built as four interleaved chains (chain
// c = i mod 4 starts at rot * step^c and advances by step^4), every float
// product and sum rounded separately (no contraction); non-finite results
// become 0.  One thread per (frame, slot, chain).
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cusat_fec.h"
#include "kernels.h"

namespace {

constexpr int kSlot = 90, kPilotBlock = 36, kSlotsPerPilot = 16;
constexpr int kPeriod = (1 << 18) - 1;       // m-sequence period
constexpr int kMaxPayload = 360 * 90 + 22 * 36;  // QPSK normal frame with pilots, the longest payload

int fail(int code, const std::string& msg)
{
    cusat::set_last_error(msg);
    return code;
}

int cuda_fail(cudaError_t e, const char* what)
{
    cusat::set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
    return CUSAT_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// PLFRAME layout from the PLS code.  Data of the standard: EN 302 307-1
// Table 12 (MODCOD field, b7 = 0), EN 302 307-2 Table 17a (S2X MODCODs,
// b7 = 1: code, bits per symbol, frame size, this project's MODCOD index)
// and Table 17b (reserved codes with a defined length), as in the
// reference's framing/plframe.cc:30-158.
struct S2xCode { uint8_t code, bits, fs, modcod; };
constexpr S2xCode kS2x[] = {
    {132, 2, 0, 33}, {134, 2, 0, 43}, {136, 2, 0, 44}, {138, 3, 0, 56}, {140, 3, 0, 57}, {142, 3, 0, 45},
    {144, 3, 0, 46}, {146, 3, 0, 47}, {148, 4, 0, 58}, {150, 4, 0, 59}, {152, 4, 0, 60}, {154, 4, 0, 48},
    {156, 4, 0, 49}, {158, 4, 0, 61}, {160, 4, 0, 50}, {162, 4, 0, 51}, {164, 4, 0, 62}, {166, 4, 0, 52},
    {168, 4, 0, 53}, {170, 4, 0, 54}, {172, 4, 0, 55}, {174, 5, 0, 63}, {178, 5, 0, 64}, {180, 5, 0, 65},
    {182, 5, 0, 66}, {184, 6, 0, 36}, {186, 6, 0, 29}, {190, 6, 0, 30}, {194, 6, 0, 31}, {198, 6, 0, 35},
    {200, 7, 0, 32}, {202, 7, 0, 34}, {204, 8, 0, 39}, {206, 8, 0, 41}, {208, 8, 0, 40}, {210, 8, 0, 38},
    {212, 8, 0, 42}, {214, 8, 0, 37}, {216, 2, 1, 0},  {218, 2, 1, 0},  {220, 2, 1, 0},  {222, 2, 1, 0},
    {224, 2, 1, 0},  {226, 2, 1, 0},  {228, 3, 1, 0},  {230, 3, 1, 0},  {232, 3, 1, 0},  {234, 3, 1, 0},
    {236, 4, 1, 0},  {238, 4, 1, 0},  {240, 4, 1, 0},  {242, 4, 1, 0},  {244, 4, 1, 0},  {246, 5, 1, 0},
    {248, 5, 1, 0},
};
struct ReservedCode { uint8_t code, bits, pilots; };
constexpr ReservedCode kReserved[] = {
    {128, 3, 0}, {130, 4, 0}, {176, 5, 0}, {177, 5, 1}, {188, 6, 0}, {189, 6, 1}, {192, 6, 0}, {193, 6, 1},
    {196, 6, 0}, {197, 6, 1}, {250, 3, 1}, {251, 4, 1}, {252, 5, 1}, {253, 6, 1}, {254, 8, 1}, {255, 10, 1},
};

struct Layout {
    int slots = 0, pilots = 0, modcod = 0, fs = 0, bits = 0, dummy = 0, reserved = 0;
    int pilot_blocks() const { return pilots && slots > 0 ? (slots - 1) / kSlotsPerPilot : 0; }
    int data() const { return kSlot * slots; }
    int payload() const { return data() + kPilotBlock * pilot_blocks(); }
};

// slots of an XFECFRAME of `bits` bits per symbol (128APSK: 6 stuffing bits
// and 12 padding symbols make 103 slots; normal frames only)
int slots_for(int bits, int fs)
{
    const int n = fs == 0 ? 64800 : 16200;
    if (bits == 7)
        return fs == 0 ? 103 : 0;
    if (bits <= 0 || n % (kSlot * bits) != 0)
        return 0;
    return n / (kSlot * bits);
}

Layout layout_of(int code)
{
    Layout l;
    if (!(code & 0x80)) {
        const int mc = code >> 2;
        l.fs = (code & 2) ? 1 : 0;
        if (mc == 0) {  // dummy PLFRAME: 36 slots, no pilots
            l.dummy = 1;
            l.slots = 36;
            return l;
        }
        const int bits = mc <= 11 ? 2 : mc <= 17 ? 3 : mc <= 23 ? 4 : mc <= 28 ? 5 : 0;
        if (!bits)
            return l;
        l.pilots = code & 1;
        l.bits = bits;
        l.slots = slots_for(bits, l.fs);
        l.modcod = mc;
        return l;
    }
    for (const ReservedCode& r : kReserved)
        if (r.code == code) {
            l.reserved = 1;
            l.pilots = r.pilots;
            l.slots = slots_for(r.bits, 0);
            return l;
        }
    for (const S2xCode& e : kS2x)
        if (e.code == (code & 0xfe)) {
            l.fs = e.fs;
            l.pilots = code & 1;
            l.bits = e.bits;
            l.slots = slots_for(e.bits, e.fs);
            l.modcod = e.modcod;
            return l;
        }
    return l;  // VL-SNR headers: length not defined here
}

// A frame that carries an XFECFRAME this project decodes: not dummy or
// reserved, a known MODCOD, and a code for its frame size (short frames only
// for the DVB-S2 MODCODs 1-28 with a short code: all but the 9/10 ones).
bool deliverable(const Layout& l)
{
    if (l.dummy || l.reserved || l.modcod == 0 || l.bits == 0 || l.slots == 0)
        return false;
    if (l.fs == 1)
        return l.modcod <= 28 && l.modcod != 11 && l.modcod != 17 && l.modcod != 23 && l.modcod != 28;
    return true;
}

// ---------------------------------------------------------------------------
// Scrambler rotation index R_n(i) = 2 z_n(i + 2^17) + z_n(i),
// z_n(i) = x(i + n) XOR y(i) (EN 302 307-1 clause 5.5.4): the two m-sequences
// are generated once, one bit per byte, over a full period.
const std::vector<uint8_t>& m_sequences()
{
    static std::vector<uint8_t> xy;
    static std::once_flag once;
    std::call_once(once, [] {
        xy.assign(2 * (size_t)kPeriod, 0);
        uint32_t x = 1, y = (1u << 18) - 1;  // bit k = sequence value at i + k
        for (int i = 0; i < kPeriod; i++) {
            xy[i] = (uint8_t)(x & 1);
            xy[kPeriod + i] = (uint8_t)(y & 1);
            const uint32_t xn = (x ^ (x >> 7)) & 1;
            const uint32_t yn = (y ^ (y >> 5) ^ (y >> 7) ^ (y >> 10)) & 1;
            x = (x >> 1) | (xn << 17);
            y = (y >> 1) | (yn << 17);
        }
    });
    return xy;
}

void rotation_index(int gold, uint8_t* r, int len)
{
    const std::vector<uint8_t>& xy = m_sequences();
    const uint8_t* x = xy.data();
    const uint8_t* y = xy.data() + kPeriod;
    int a = gold % kPeriod, b = 0, c = (gold + (1 << 17)) % kPeriod, d = 1 << 17;
    for (int i = 0; i < len; i++) {
        r[i] = (uint8_t)(2 * (x[c] ^ y[d]) + (x[a] ^ y[b]));
        if (++a == kPeriod) a = 0;
        if (++b == kPeriod) b = 0;
        if (++c == kPeriod) c = 0;
        if (++d == kPeriod) d = 0;
    }
}

// ---------------------------------------------------------------------------
struct PlFrameDev {
    const float2* payload;
    float2* data;
    const float4* slot_rot;  // per slot {rot re, rot im, step re, step im}, or nullptr
    int slots, pilot_blocks, table, pad;
};

__device__ __forceinline__ float cmul_re(float ar, float ai, float br, float bi)
{
    return __fsub_rn(__fmul_rn(ar, br), __fmul_rn(ai, bi));
}

__device__ __forceinline__ float cmul_im(float ar, float ai, float br, float bi)
{
    return __fadd_rn(__fmul_rn(ar, bi), __fmul_rn(ai, br));
}

__global__ void __launch_bounds__(128) pl_extract_kernel(const PlFrameDev* frames, const uint8_t* tables, int table_len)
{
    const PlFrameDev f = frames[blockIdx.y];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int s = t >> 2, c = t & 3;
    if (s >= f.slots)
        return;
    const int off = s * kSlot + min(s / kSlotsPerPilot, f.pilot_blocks) * kPilotBlock;
    float rr = 1.0f, ri = 0.0f, sr = 1.0f, si = 0.0f;
    if (f.slot_rot) {
        const float4 q = f.slot_rot[s];
        rr = q.x;
        ri = q.y;
        sr = q.z;
        si = q.w;
    }
    // chain c starts at rot * step^c, built by repeated products as the
    // reference does; each chain advances by step^4
    float cr = rr, ci = ri;
    for (int k = 1; k <= c; k++) {
        const float nr = cmul_re(cr, ci, sr, si);
        ci = cmul_im(cr, ci, sr, si);
        cr = nr;
    }
    float pr = sr, pi = si;
    for (int k = 1; k < 4; k++) {
        const float nr = cmul_re(pr, pi, sr, si);
        pi = cmul_im(pr, pi, sr, si);
        pr = nr;
    }
    const uint8_t* rix = tables + (size_t)f.table * table_len + off;
    const float2* in = f.payload + off;
    float2* out = f.data + (size_t)s * kSlot;
    for (int i = c; i < kSlot; i += 4) {
        const float2 a = in[i];
        const int q = rix[i] & 3;
        // e^{-j R pi/2}: (1, 0), (0, -1), (-1, 0), (0, 1)
        const float br = q == 0 ? 1.0f : q == 2 ? -1.0f : 0.0f;
        const float bi = q == 1 ? -1.0f : q == 3 ? 1.0f : 0.0f;
        const float xr = cmul_re(a.x, a.y, br, bi), xi = cmul_im(a.x, a.y, br, bi);
        float vr = cmul_re(xr, xi, cr, ci), vi = cmul_im(xr, xi, cr, ci);
        if (i < kSlot - 2) {  // the chains advance once per group of four symbols
            const float nr = cmul_re(cr, ci, pr, pi);
            ci = cmul_im(cr, ci, pr, pi);
            cr = nr;
        }
        if (!isfinite(vr) || !isfinite(vi))
            vr = vi = 0.0f;
        out[i] = make_float2(vr, vi);
    }
}

}  // namespace

struct cusat_pl_extractor {
    std::vector<int32_t> golds;   // scrambling codes with a table on the device
    uint8_t* tables = nullptr;    // [codes][kMaxPayload] rotation indices
    int max_frames = 0;
    PlFrameDev* h_frames = nullptr;  // pinned staging
    PlFrameDev* d_frames = nullptr;
    cudaEvent_t copied = nullptr;    // the last call's descriptor copy
    bool pending = false;
};

namespace {

void release(cusat_pl_extractor* x)
{
    if (!x)
        return;
    if (x->tables) cudaFree(x->tables);
    if (x->d_frames) cudaFree(x->d_frames);
    if (x->h_frames) cudaFreeHost(x->h_frames);
    if (x->copied) cudaEventDestroy(x->copied);
    delete x;
}

}  // namespace

extern "C" {

int cusat_pl_layout(int pls_code, int32_t* out)
{
    if (!out || pls_code < 0 || pls_code > 255)
        return fail(CUSAT_ERR_ARG, "PLS code outside 0..255 or null output");
    const Layout l = layout_of(pls_code);
    out[0] = l.slots;
    out[1] = l.pilots;
    out[2] = l.pilot_blocks();
    out[3] = l.data();
    out[4] = l.slots ? l.payload() : 0;
    out[5] = l.modcod;
    out[6] = l.fs;
    out[7] = l.bits;
    out[8] = l.dummy;
    out[9] = deliverable(l) ? 1 : 0;
    out[10] = l.reserved;
    return CUSAT_OK;
}

int cusat_pl_rotation_index(int gold, uint8_t* r, int len)
{
    if (!r || len < 0 || gold < 0 || gold >= kPeriod - 1)
        return fail(CUSAT_ERR_ARG, "scrambling code outside 0..262141 or bad buffer");
    rotation_index(gold, r, len);
    return CUSAT_OK;
}

int cusat_pl_extractor_create(const int32_t* gold_codes, int n_codes, int max_frames, cusat_pl_extractor** out)
{
    if (!out || !gold_codes || n_codes <= 0 || n_codes > 4096 || max_frames <= 0 || max_frames > 65535)
        return fail(CUSAT_ERR_ARG, "invalid PL extractor arguments");
    *out = nullptr;
    int n_dev = 0;
    if (cudaGetDeviceCount(&n_dev) != cudaSuccess || n_dev == 0)
        return fail(CUSAT_ERR_NO_DEVICE, "no CUDA device");
    cusat_pl_extractor* x = new cusat_pl_extractor();
    x->max_frames = max_frames;
    std::vector<uint8_t> h((size_t)n_codes * kMaxPayload);
    for (int k = 0; k < n_codes; k++) {
        if (gold_codes[k] < 0 || gold_codes[k] >= kPeriod - 1) {
            release(x);
            return fail(CUSAT_ERR_ARG, "scrambling code outside 0..262141");
        }
        x->golds.push_back(gold_codes[k]);
        rotation_index(gold_codes[k], h.data() + (size_t)k * kMaxPayload, kMaxPayload);
    }
    cudaError_t e = cudaMalloc(&x->tables, h.size());
    if (e == cudaSuccess)
        e = cudaMemcpy(x->tables, h.data(), h.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMalloc(&x->d_frames, (size_t)max_frames * sizeof(PlFrameDev));
    if (e == cudaSuccess)
        e = cudaMallocHost(&x->h_frames, (size_t)max_frames * sizeof(PlFrameDev));
    if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(&x->copied, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        release(x);
        return cuda_fail(e, "PL extractor buffers");
    }
    *out = x;
    return CUSAT_OK;
}

void cusat_pl_extractor_destroy(cusat_pl_extractor* x) { release(x); }

int cusat_pl_extract(cusat_pl_extractor* x, const cusat_pl_frame* frames, int n, void* stream)
{
    if (!x || !frames || n <= 0 || n > x->max_frames)
        return fail(CUSAT_ERR_ARG, "frames outside 1..max_frames");
    // the staging buffer is read by the previous call's copy
    if (x->pending) {
        const cudaError_t e = cudaEventSynchronize(x->copied);
        if (e != cudaSuccess)
            return cuda_fail(e, "cudaEventSynchronize");
        x->pending = false;
    }
    int max_slots = 0;
    for (int f = 0; f < n; f++) {
        const cusat_pl_frame& fr = frames[f];
        if (!fr.payload || !fr.data)
            return fail(CUSAT_ERR_ARG, "null frame buffer");
        if (fr.pls_code < 0 || fr.pls_code > 255)
            return fail(CUSAT_ERR_ARG, "PLS code outside 0..255");
        const Layout l = layout_of(fr.pls_code);
        if (!deliverable(l))
            return fail(CUSAT_ERR_UNSUPPORTED, "PLS code carries no decodable XFECFRAME");
        const auto it = std::find(x->golds.begin(), x->golds.end(), fr.gold);
        if (it == x->golds.end())
            return fail(CUSAT_ERR_ARG, "scrambling code not given to cusat_pl_extractor_create");
        PlFrameDev& d = x->h_frames[f];
        d.payload = reinterpret_cast<const float2*>(fr.payload);
        d.data = reinterpret_cast<float2*>(fr.data);
        d.slot_rot = reinterpret_cast<const float4*>(fr.slot_rot);
        d.slots = l.slots;
        d.pilot_blocks = l.pilot_blocks();
        d.table = (int)(it - x->golds.begin());
        d.pad = 0;
        max_slots = std::max(max_slots, l.slots);
        if ((reinterpret_cast<uintptr_t>(fr.payload) & 7) || (reinterpret_cast<uintptr_t>(fr.data) & 7) ||
            (reinterpret_cast<uintptr_t>(fr.slot_rot) & 15))
            return fail(CUSAT_ERR_ARG, "payload/data need 8-byte, slot rotations 16-byte alignment");
    }
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(x->d_frames, x->h_frames, (size_t)n * sizeof(PlFrameDev),
                                    cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaEventRecord(x->copied, s);
    if (e != cudaSuccess)
        return cuda_fail(e, "descriptor copy");
    x->pending = true;
    const dim3 grid((unsigned)((max_slots * 4 + 127) / 128), (unsigned)n);
    pl_extract_kernel<<<grid, 128, 0, s>>>(x->d_frames, x->tables, kMaxPayload);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return cuda_fail(e, "PL extract launch");
    return CUSAT_OK;
}

}  // extern "C"
