// fluid3d_access.h -- what other parts of the library (the adjoint) may reach inside a 3D
// fluid handle; implemented in fluid3d.cu.
#pragma once

#include "fluid3d_kernels.cuh"

namespace gbsph {

struct FluidAccess {
    float4 *pos, *vel, *force, *spos, *svel;
    uint32_t *index, *keys;
    size_t n;
    bool has_hook, compiled;
};
// Validates the parameters, makes the cell table match them, fills `a` and the step's kernel
// parameters.
int fluid3d_access(gbsph_fluid3d_t h, FluidAccess* a, KParams* kp);
// While `rec` is set, every step writes each particle's force after the clip box into it;
// while `rec_nbr` / `rec_cnt` are set, the brick kernels' neighbour lists into the slot
// *rec_slot of them (KParams::rec_nbr).
void fluid3d_set_record(gbsph_fluid3d_t h, float4* rec, uint32_t* rec_nbr = nullptr, uint32_t* rec_cnt = nullptr,
                        const uint32_t* rec_slot = nullptr, uint32_t rec_n4 = 0);

}  // namespace gbsph
