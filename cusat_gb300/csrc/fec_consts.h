// Constants shared by the host plan builder and the kernels.
#pragma once

#include <stdint.h>

namespace cusat {

constexpr int kM = 360;            // circulant size of every DVB-S2/S2X code
constexpr int kLaneThreads = 384;  // 12 warps per decoding lane (360 check rows)
constexpr int kMaxStage = 8;       // guest delta rows per schedule step
constexpr int kBig = 1 << 20;      // |extrinsic| of an absent edge

// Circulant descriptor word of one (layer, slot):
//   bits  0-15 base = information group * 360
//   bits 16-24 shift s: check j of the layer reads bit base + (j - s) mod 360
//   bits 25-26 role: 0 plain, 1 owner, 2 guest (shared variable node in a step)
//   bits 27-29 guest: stage row; owner: first stage row of its guests
//   bits 30-31 owner: number of guests - 1
constexpr uint32_t kRolePlain = 0, kRoleOwner = 1, kRoleGuest = 2;

}  // namespace cusat
