// Constants shared by the host plan builder and the kernels.
#pragma once

#include <stdint.h>

namespace cusat {

constexpr int kM = 360;            // circulant size of every DVB-S2/S2X code
constexpr int kLaneThreads = 384;  // 12 warps per decoding lane (360 check rows)
constexpr int kMaxStage = 16;      // stage rows (guest deltas + owner values) per step
constexpr int kBig = 1 << 20;      // |extrinsic| of an absent edge

// Slot descriptor of one (layer, circulant), uint2:
//   x = byte offset in the APP of the circulant's first bit (2 * group * 360)
//   y bits 0-15  r = (360 - shift) mod 360: check j of the layer reads bit
//                (j + r) mod 360 of the group
//   y bits 16-23 stage row (guest and owner slots)
// The circulants of a layer are ordered plain, guest, owner: a plain
// circulant is the only writer of its bits in the step; when several
// circulants of one step share an information group, the first is the owner
// (its updated APP goes to a stage row) and the others are guests (their
// message deltas go to stage rows); after a barrier the owner items of the
// step add the rows up.  Owner item, uint2: x = byte offset of the group in
// the APP, y = owner row | first guest row << 8 | guests << 16.

}  // namespace cusat
