// Device view of the structures a server keeps resident between evaluations.
#pragma once

#include "common.cuh"

namespace nnapgb {

// One resident structure as one tick of the server sees it.  The Verlet rows were
// built at rc + skin from the positions of the last rebuild; kb holds, per atom, the
// lattice counts that wrapping subtracted at that rebuild (floor of the direct
// coordinates), so a later wrap that moves an atom across the box is turned into the
// matching change of every pair image.
struct SlotDev {
    uint64_t* vkey;    // [n*Mv] (local j << 32) | packed image at the rebuild
    uint16_t* vgrp;    // [n*Mv] cell-offset group on the rebuild's cell grid
    int* vcnt;         // [n] Verlet count (above Mv when the rebuild overflowed)
    int4* kb;          // [n] wrap counts at the rebuild
    const int* type;   // [n] species (1-based)
    int a0, n;         // atom range of the structure in this tick's batch
};

}  // namespace nnapgb
