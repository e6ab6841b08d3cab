// hgpu_spawn_rdm.cu -- the spawning kernels that also record replica 2-RDM
// spawns (spawn_rdm, src/spawning.F90:588-676), in a translation unit of their
// own: the kernels of calculations without density_matrices carry none of
// their code, and the two sets compile in parallel.
#include "hgpu_spawn.cuh"

namespace hgpu {

template <int W>
static void spawn_rdm_w(const DevBuffers &b, int R, int kind, int precision, int cur, size_t sm, cudaStream_t st) {
#define HGPU_SPAWN_RDM(KK)                                                  \
    do {                                                                    \
        if (precision == HGPU_PREC_MIXED)                                   \
            launch_spawn_kernels<W, KK, float, true>(b, R, cur, sm, st);    \
        else                                                                \
            launch_spawn_kernels<W, KK, double, true>(b, R, cur, sm, st);   \
    } while (0)
    if (kind == kKindHeatBath) HGPU_SPAWN_RDM(kKindHeatBath);
    else if (kind == kKindHeatBathUniform) HGPU_SPAWN_RDM(kKindHeatBathUniform);
    else if (kind == kKindReadInNoRenorm) HGPU_SPAWN_RDM(kKindReadInNoRenorm);
    else if (kind == kKindPowerPitzerOcc)
        launch_spawn_kernels<W, kKindPowerPitzerOcc, double, true>(b, R, cur, sm, st);
    else if (kind == kKindPowerPitzerRef)
        launch_spawn_kernels<W, kKindPowerPitzerRef, double, true>(b, R, cur, sm, st);
    else HGPU_SPAWN_RDM(HGPU_SYS_READ_IN);
#undef HGPU_SPAWN_RDM
}

void launch_spawn_rdm(const DevBuffers &b, int W, int R, int kind, int precision, int cur, size_t sm,
                      cudaStream_t st) {
    if (W == 1) spawn_rdm_w<1>(b, R, kind, precision, cur, sm, st);
    else spawn_rdm_w<2>(b, R, kind, precision, cur, sm, st);
}

}  // namespace hgpu
