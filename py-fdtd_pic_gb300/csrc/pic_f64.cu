// FP64 instantiation of the PIC step (built with -fmad=false, like the FDTD parity path).
#include "pic_kernel.cuh"

namespace fdtdpic {

int run_pic_f64(const FdtdInstance &h, const BatchArgs<double> &fa, const PicBeam &bm,
                int32_t *cell, double *frac, double *ux, double *uz, int32_t *id, double *jx,
                double *jz, double *hyp, unsigned char *scratch, int32_t *status, FdtdPicTiming *timing,
                cudaStream_t st, bool allow_graphs)
{
    return launch_pic<double>(8, h, fa, bm, cell, frac, ux, uz, id, jx, jz, hyp, scratch, status, timing, st,
                          allow_graphs);
}

}  // namespace fdtdpic

#include "pic_tiled.cuh"

namespace fdtdpic {

int run_pic_tiled_f64(const FdtdInstance &h, const BatchArgs<double> &fa, const PicBeam &bm,
                      const TileGeom &g, int32_t *cell, double *frac, double *ux, double *uz, int32_t *id,
                      double *jx, double *jz, double *hyp, unsigned char *scratch, int32_t *status,
                      FdtdPicTiming *timing, cudaStream_t st)
{
    return launch_pic_tiled<double>(sizeof(double), h, fa, bm, g, cell, frac, ux, uz, id, jx, jz, hyp,
                                 scratch, status, timing, st);
}

}  // namespace fdtdpic

#include "pic_pass.cuh"

namespace fdtdpic {

int run_pic_pass_f64(const FdtdInstance &h, const BatchArgs<double> &fa, const PicBeam &bm,
                     const PassGeom &g, int32_t *cell, double *frac, double *ux, double *uz, int32_t *id,
                     double *jx, double *jz, double *hyp, unsigned char *scratch, int32_t *status,
                     FdtdPicTiming *timing, cudaStream_t st)
{
    return launch_pic_pass<double>(sizeof(double), h, fa, bm, g, cell, frac, ux, uz, id, jx, jz, hyp,
                                scratch, status, timing, st);
}

}  // namespace fdtdpic
