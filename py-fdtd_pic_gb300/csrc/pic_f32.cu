// FP32 instantiation of the PIC step.
#include "pic_kernel.cuh"

namespace fdtdpic {

int run_pic_f32(const FdtdInstance &h, const BatchArgs<float> &fa, const PicBeam &bm,
                int32_t *cell, float *frac, float *ux, float *uz, int32_t *id, float *jx,
                float *jz, float *hyp, unsigned char *scratch, int32_t *status, FdtdPicTiming *timing,
                cudaStream_t st, bool allow_graphs)
{
    return launch_pic<float>(4, h, fa, bm, cell, frac, ux, uz, id, jx, jz, hyp, scratch, status, timing, st,
                          allow_graphs);
}

}  // namespace fdtdpic

#include "pic_tiled.cuh"

namespace fdtdpic {

int run_pic_tiled_f32(const FdtdInstance &h, const BatchArgs<float> &fa, const PicBeam &bm,
                      const TileGeom &g, int32_t *cell, float *frac, float *ux, float *uz, int32_t *id,
                      float *jx, float *jz, float *hyp, unsigned char *scratch, int32_t *status,
                      FdtdPicTiming *timing, cudaStream_t st)
{
    return launch_pic_tiled<float>(sizeof(float), h, fa, bm, g, cell, frac, ux, uz, id, jx, jz, hyp,
                                 scratch, status, timing, st);
}

}  // namespace fdtdpic

#include "pic_pass.cuh"

namespace fdtdpic {

int run_pic_pass_f32(const FdtdInstance &h, const BatchArgs<float> &fa, const PicBeam &bm,
                     const PassGeom &g, int32_t *cell, float *frac, float *ux, float *uz, int32_t *id,
                     float *jx, float *jz, float *hyp, unsigned char *scratch, int32_t *status,
                     FdtdPicTiming *timing, cudaStream_t st)
{
    return launch_pic_pass<float>(sizeof(float), h, fa, bm, g, cell, frac, ux, uz, id, jx, jz, hyp,
                                scratch, status, timing, st);
}

}  // namespace fdtdpic
