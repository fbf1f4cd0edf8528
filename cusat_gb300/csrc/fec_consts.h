// Constants shared by the host plan builder and the kernels.
#pragma once

#include <stdint.h>

namespace cusat {

constexpr int kM = 360;            // circulant size of every DVB-S2/S2X code
// Threads of a decoding lane (one per check row of a layer, 360, plus idle
// threads up to a warp boundary when the CTA has one lane): two lanes share
// a warp (720 threads, 23 warps); one lane keeps 12 whole warps, measured
// faster on GB300 than 360 threads in 12 warps with the last one partial.
#ifdef __CUDACC__
__host__ __device__
#endif
constexpr int lane_threads(int lanes) { return lanes == 2 ? 360 : 384; }
constexpr int kMaxStage = 16;      // stage rows per step (one per circulant of a shared group)
constexpr int kBig = 1 << 20;      // |extrinsic| of an absent edge

// Where the next step's message rows wait: shared memory (per-thread
// asynchronous copies) or registers (loads one step ahead).  Measured per
// kernel class on GB300: shared memory wins only for 8 and 9 slots x 2
// lanes; the other classes lose more L1 (their register spills live there)
// than they gain in registers.
#ifdef __CUDACC__
__host__ __device__
#endif
constexpr bool stage_rows_in_smem(int cmax, int lanes) { return (cmax == 8 || cmax == 9) && lanes == 2; }

// 32-bit words of one check row of messages in the one-frame kernel: one
// byte per edge (cmax + 2 edges), rounded up to 4, 8, 12, 16 or 32 bytes
// (one load or store per row, three for 12), so that the rows of the
// resident CTAs stay in L2 (normal rate 1/4, 48,600 checks: 4 bytes instead
// of 16, 30 instead of 118 MB for 152 CTAs).  Rows staged in shared memory
// stay 16 bytes: one 16-byte asynchronous copy; three 4-byte ones measured
// 12 % slower on the 9-slot two-lane class.
#ifdef __CUDACC__
__host__ __device__
#endif
constexpr int row_words(int cmax, int lanes)
{
    return stage_rows_in_smem(cmax, lanes) ? 4
           : cmax + 2 <= 4                 ? 1
           : cmax + 2 <= 8                 ? 2
           : cmax + 2 <= 12                ? 3
           : cmax + 2 <= 16                ? 4
                                           : 8;
}

// Slot descriptor of one (layer, circulant slot), uint4:
//   x = byte offset in shared memory of the circulant's first bit
//   y = r = (360 - shift) mod 360: check j of the layer reads bit
//       (j + r) mod 360 of the group
//   z = byte offset from a bit's APP slot to where its update is stored:
//       0 when the circulant is the only writer of its group in the step;
//       otherwise the bit's entry in this circulant's stage row
//   w = kind: 0 plain, 1 staged, 2 absent (the layer has fewer circulants
//       than the kernel's slots: reads a region of +32640, writes a junk
//       region, contributes nothing)
// x and z of staged and absent slots are relative to the stage/dummy
// regions and are rebased when a kernel copies the table to shared memory
// (y becomes 2 r there; the frame-pair kernel also doubles the APP offsets
// and places the stage rows in its own sets).
// When several circulants of one step share an information group, each
// writes its updated bits to its own int16 stage row, and a group item of
// the step (uint2: x = byte offset of the group, y = first row | rows << 8)
// later stores APP + sum over the rows of (row - APP) (the deltas in the
// saturating path).  The completion runs at the start of the next step when
// that step does not touch the group, otherwise after a mid-step barrier.
constexpr uint32_t kSlotPlain = 0, kSlotStaged = 1, kSlotAbsent = 2;
constexpr int kStageSets = 2;  // stage rows alternate between even and odd steps
constexpr uint8_t kConfDefer = 1, kConfMid = 2;

}  // namespace cusat
