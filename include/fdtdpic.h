/*
 * fdtdpic: GB300 (sm_103a) implementation of the 1D FDTD/PIC time-stepping path of
 * fraserac/Py-FDTD_PIC.  Plain C ABI: raw device pointers, sizes, a CUDA stream, int status.
 *
 * Every entry point returns FDTDPIC_OK (0) or a negative FDTDPIC_ERR_* code; none throws.
 * Pointers named d_* are caller-owned DEVICE memory (e.g. torch tensors' data_ptr()); the calls
 * are asynchronous on the given stream unless stated.  A handle-free design: no call keeps state
 * between calls except the per-device function attributes set on first use.
 *
 * Reference interfaces replaced (file:line in fraserac/Py-FDTD_PIC):
 *   fdtd1d_run_batch / fdtd1d_run_global
 *       the per-step loops of Solver_Engine.IntegratorNL1D (Solver_Engine.py:220-271),
 *       IntegratorLinLor1D (:275-371, one call per pass) and IntegratorFreeSpace1D (:142-215),
 *       i.e. BaseFDTD11.ADE_ExUpdate (BaseFDTD11.py:664), CPML_Psi_e_Update (:365),
 *       ADE_DxUpdate (:751), AcubicFinder/Nonlin_Cubic_Solver (:803-853) with
 *       CubicEquationSolver.solve (CubicEquationSolver.py:29), NonLinExUpdate (:859),
 *       ADE_TempPolCurr/ADE_PolarisationCurrent_Ex (:487, :610), ADE_ExCreate (:713),
 *       ADE_HyUpdate (:641), CPML_Psi_m_Update (:382), probeSim (Solver_Engine.py:16),
 *       vidMake (Solver_Engine.py:57).
 *   fdtdpic_cubic_root0
 *       Re(CubicEquationSolver.solve(a,b,c,d)[0]) as kept by Nonlin_Cubic_Solver
 *       (BaseFDTD11.py:838), batched.
 */
#ifndef FDTDPIC_H
#define FDTDPIC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *fdtdpic_stream_t; /* == cudaStream_t */

#define FDTDPIC_ABI_VERSION 2

#define FDTDPIC_OK 0
#define FDTDPIC_ERR_ARG (-1)     /* invalid argument (sizes, pointers, modes) */
#define FDTDPIC_ERR_OOM (-2)     /* an instance does not fit the chosen path's memory */
#define FDTDPIC_ERR_TIMEOUT (-3) /* a bounded device-side wait gave up */
#define FDTDPIC_ERR_NUMERIC (-4) /* non-finite state detected (see status words) */
#define FDTDPIC_ERR_CUDA (-5)    /* a CUDA runtime call failed */
#define FDTDPIC_ERR_NODEV (-6)   /* no usable sm_103 device */

#define FDTD_MODE_FREESPACE 0 /* IntegratorFreeSpace1D */
#define FDTD_MODE_LINLOR 1    /* IntegratorLinLor1D (one pass per instance) */
#define FDTD_MODE_KERR 2      /* IntegratorNL1D */

#define FDTDPIC_F64 8 /* precision argument: FP64 state (parity path) */
#define FDTDPIC_F32 4 /* FP32 state, FP64 near-degenerate cubic solves */

/* Size limits: the kernels index cells and particles with 32-bit integers, with headroom for
 * per-launch offsets.  Every entry point refuses a larger FdtdInstance.nz, and fdtdpic_run and
 * fdtdpic_slot_check a larger beam, with FDTDPIC_ERR_ARG before any device work
 * (fdtdpic_run_noalloc's 24 MiB scratch refuses such a beam first, with FDTDPIC_ERR_OOM). */
#define FDTDPIC_MAX_CELLS (1 << 30)     /* FdtdInstance.nz */
#define FDTDPIC_MAX_PARTICLES (1 << 30) /* PicBeam.n_part, FdtdSlot.n_part */

/* Per-instance status bits (d_status[i]) */
#define FDTD_STATUS_NONFINITE 1 /* Ex or Hy not finite at the end of the call */
#define FDTD_STATUS_SKIPPED 2   /* instance larger than smem_bytes: not run */
#define FDTD_STATUS_TIMEOUT 4   /* beam step, tiled path: a bounded wait gave up */
#define FDTD_STATUS_OVERFLOW 8  /* beam step, tiled or pass path: a tile, migrant or segment
                                   buffer overflowed */
#define FDTD_STATUS_BOUNDS 16   /* the index-checking debug build (libfdtdpic_bounds.so) found an
                                   index outside its buffer and skipped the access */

/* PML coefficient table: per instance FDTD_TAB_ROWS rows x (2*pml+1) columns of doubles.
 * Column c <= pml is cell c; column c > pml is cell nz+1-pml+(c-pml-1). */
#define FDTD_TAB_BEX 0
#define FDTD_TAB_CEX 1
#define FDTD_TAB_CB 2
#define FDTD_TAB_BMY 3
#define FDTD_TAB_CMY 4
#define FDTD_TAB_C2 5
#define FDTD_TAB_DENE 6
#define FDTD_TAB_DENH 7
#define FDTD_TAB_ROWS 8

/* State buffer: per instance FDTD_STATE_ARRAYS arrays of nz+1 elements of the precision's type,
 * in this order, starting at state_offset. */
#define FDTD_ST_EX 0
#define FDTD_ST_HY 1
#define FDTD_ST_DX 2
#define FDTD_ST_P 3     /* polarisationCurr */
#define FDTD_ST_PPREV 4 /* tempVarPol (P one step back) */
#define FDTD_ST_PSIE 5
#define FDTD_ST_PSIH 6
#define FDTD_ST_A 7 /* Acubic */
#define FDTD_STATE_ARRAYS 8

/* One 1D grid ("instance").  Field names follow the reference's Params/Variables. */
typedef struct FdtdInstance {
    int32_t nz;            /* Params.Nz; arrays have nz+1 cells */
    int32_t n_steps;       /* Params.timeSteps (length of the source arrays) */
    int32_t step_begin;    /* first step this call runs (0 for a fresh run) */
    int32_t step_end;      /* one past the last step this call runs */
    int32_t pml;           /* Params.pmlWidth */
    int32_t cpml_lo;       /* Params.CPMLXm */
    int32_t cpml_hi;       /* Params.CPMLXp */
    int32_t front;         /* Params.materialFrontEdge */
    int32_t rear;          /* Params.materialRearEdge */
    int32_t nzsrc;         /* Params.nzsrc */
    int32_t tfsf;          /* Params.TFSF */
    int32_t mode;          /* FDTD_MODE_* */
    int32_t pol_active;    /* LinLor: 1 runs the polarisation update (pass i==1) */
    int32_t resume;        /* 1: start from the state buffer, 0: from zero fields (FieldInit) */
    int32_t hist_interval; /* Params.vidInterval; 0 disables snapshots */
    int32_t hist_rows;     /* rows of this instance's snapshot buffer */
    int32_t probe_cell[2]; /* cells sampled after every step ... */
    int32_t probe_lo[2];   /* ... for steps probe_lo <= t <= probe_hi (inclusive) */
    int32_t probe_hi[2];
    double ue;       /* UpExMat outside the slab (CharImp * courantNo) */
    double ue_slab;  /* UpExMat inside [front, rear) (free space: divided by epsRe) */
    double uh;       /* UpHyMat outside the slab ((1/CharImp) * courantNo) */
    double uh_slab;  /* UpHyMat inside the slab */
    double dtdz;     /* delT/dz */
    double eps0;     /* permit_0 */
    double sc;       /* courantNo: the source is added as Exs[t]/sc, Hys[t]/sc */
    double pol_a, pol_b, pol_c;    /* ADE_PolarisationCurrent_Ex's A, B, C */
    double kerr_a, kerr_b, kerr_c; /* AcubicFinder's cub, qua, one */
    double nl_e0;    /* permit_0 * Re(sqrt(1.2)) (NonLinExUpdate) */
    double nl_e0chi; /* permit_0 * chi3Stat */
    int64_t pml_offset;   /* doubles into d_pml_tab */
    int64_t src_offset;   /* doubles into d_src: Exs[n_steps] then Hys[n_steps] */
    int64_t probe_offset; /* elements into d_probe: [n_steps][2] */
    int64_t state_offset; /* elements into d_state: FDTD_STATE_ARRAYS x (nz+1) */
    int64_t hist_offset;  /* elements into d_hist: [hist_rows][nz+1] */
    int64_t srcs_offset;  /* doubles into d_src: Exs[t]/sc then Hys[t]/sc (n_steps each), the
                             source divided by courantNo ahead of time (the same correctly rounded
                             FP64 quotients the kernels would form); -1: divide on the device */
} FdtdInstance;

/* ---- library ---------------------------------------------------------------------------- */
int fdtdpic_abi_version(void);
const char *fdtdpic_strerror(int code);
/* Writes sizeof(FdtdInstance) then the byte offset of each field, in declaration order, into
 * out[0..n); returns the number of values available.  Lets a binding verify its struct layout. */
int fdtdpic_instance_layout(int64_t *out, int n);
/* SM count and the dynamic shared memory (bytes) one instance needs on the resident path
 * (0 when it does not fit); host-only, no device memory touched. */
int fdtdpic_device_sms(int *sms);
int64_t fdtd1d_resident_smem_bytes(const FdtdInstance *inst, int precision);

/* ---- FDTD ------------------------------------------------------------------------------ */
/* Run steps [step_begin, step_end) of n_inst instances in one launch.  Each CTA owns one
 * instance at a time with its fields resident in shared memory and pulls the next instance
 * index from d_queue (one int32 of caller scratch, reset by this call) in the order d_order
 * (n_inst indices; NULL = 0..n_inst-1).  smem_bytes is the dynamic shared memory per CTA, at
 * least the largest fdtd1d_resident_smem_bytes of the batch (an instance that needs more is
 * skipped and flagged FDTD_STATUS_SKIPPED; above the device limit: FDTDPIC_ERR_OOM).
 * grid_ctas <= 0 picks the
 * occupancy-limited grid.  d_probe rows outside an instance's probe windows are not written;
 * d_hist/d_status/d_fallbacks may be NULL.  d_fallbacks[i] counts the FP32 path's cubic solves
 * redone in FP64. */
int fdtd1d_run_batch(int precision, int n_inst, const FdtdInstance *d_inst, const int32_t *d_order,
                     const double *d_pml_tab, const double *d_src, void *d_state, void *d_probe,
                     void *d_hist, int32_t *d_queue, int32_t *d_status, int32_t *d_fallbacks,
                     int64_t smem_bytes, int threads_per_cta, int grid_ctas,
                     fdtdpic_stream_t stream);

/* Same steps for ONE instance of any size: fields stay in d_state (global memory) and every
 * step is two grid-wide launches (E phase, H phase).  h_inst is the host copy of d_inst[0];
 * the call loops over steps on the host side and is asynchronous on the stream. */
int fdtd1d_run_global(int precision, const FdtdInstance *h_inst, const FdtdInstance *d_inst,
                      const double *d_pml_tab, const double *d_src, void *d_state, void *d_probe,
                      void *d_hist, int32_t *d_status, int32_t *d_fallbacks,
                      fdtdpic_stream_t stream);

/* Re(roots[0]) of n cubics a*x^3+b*x^2+c*x+d with the reference's closed form, in FP64.
 * d_coef: n x 4 doubles (a,b,c,d); d_out: n doubles. */
int fdtdpic_cubic_root0(int n, const double *d_coef, double *d_out, fdtdpic_stream_t stream);

/* ---- reflection vs frequency ---------------------------------------------------------------
 * The reference turns probe traces into a reflection coefficient with an FFT and a peak-bin
 * ratio (TransformHandler.RefTester, TransformHandler.py:34-78; MasterController.results,
 * MasterController.py:485-500).  Here every requested frequency is a direct DFT of every trace,
 * batched: X[r, f] = sum_n x[r, n] exp(-2 pi i f_k n dt), FP32 products, FP64 accumulation of
 * 64-step chunks. */
/* Bytes of the twiddle table for F frequencies and S samples (F x S float2). */
int64_t fdtdpic_dft_twiddle_bytes(int F, int S);
/* Fill the twiddle table (phase reduced in FP64, values in FP32); d_freqs: F doubles [Hz]. */
int fdtdpic_dft_twiddles(const double *d_freqs, int F, int S, double dt, void *d_tw,
                         fdtdpic_stream_t stream);
/* X (R x F complex, as interleaved doubles) of R traces of S samples.  Trace r, sample n is
 * element (r / rp) * ldp + (r % rp) * sp + n * sn of d_traces (FDTDPIC_F32 or FDTDPIC_F64); the
 * probe buffer of a batch with equal step counts is read in place with rp = 2, ldp = 2 S,
 * sp = 1, sn = 2. */
int fdtdpic_dft_probes(int precision, const void *d_traces, int R, int S, int rp, int64_t ldp,
                       int64_t sp, int64_t sn, const void *d_tw, int F, double *d_out,
                       fdtdpic_stream_t stream);
/* The same X on the tensor cores (tcgen05, sm_103a): split-BF16x3 products (about 16
 * significant bits each) with FP32 sums over 1024-step groups in tensor memory and compensated
 * FP32 sums (an error-free two-sum into a float pair, ~48 bits) across groups.  The operands are first packed into BF16 tiles in d_scratch (16-byte aligned,
 * fdtdpic_dft_tc_scratch_bytes(R, S, F) bytes).  d_err (one int32, caller-zeroed) is set
 * non-zero if a bounded wait for the copies or the tensor cores gave up (the affected outputs
 * are then not written). */
int64_t fdtdpic_dft_tc_scratch_bytes(int R, int S, int F);
int fdtdpic_dft_probes_tc(int precision, const void *d_traces, int R, int S, int rp, int64_t ldp,
                          int64_t sp, int64_t sn, const void *d_tw, int F, double *d_out,
                          void *d_scratch, int64_t scratch_bytes, int32_t *d_err,
                          fdtdpic_stream_t stream);
/* |R(f)| = |X[2p+1, f]| / |X[2p, f]| for n_pairs trace pairs (0 where |X[2p, f]| = 0). */
int fdtdpic_reflection_ratio(const double *d_X, int n_pairs, int F, double *d_ratio,
                             fdtdpic_stream_t stream);

/* ---- FDTD + electron-beam PIC -------------------------------------------------------------
 * Replaces the reference's Jx hook (MasterController.py:93,159; the -Jx term of ADE_ExUpdate,
 * BaseFDTD11.py:667), which the reference never fills; the beam model has no reference code.
 * Particles: position = cell (int32) + frac in [0,1) in units of dz; momentum u/c = gamma v/c
 * (ux, uz).  Each step: gather E^t and B^t = -mu0 (Hy + Hyp)/2 by CIC, relativistic Boris push,
 * Jx deposited by CIC at the half-step midpoint, Jz charge-conserving on half nodes, periodic
 * wrap into [clo, chi); then the field step of the instance's mode with -Jx in the Ex (and slab
 * Dx) update.  Deposits are exact int64 fixed-point sums (scale jscale), so results do not depend
 * on particle order or thread scheduling; particles are re-binned by cell every sort_every
 * steps so each CTA's deposits stay in a small shared-memory window. */
/* PicBeam.path: the low bits select the path (FDTDPIC_PATH_MODE); FDTDPIC_PATH_CELLS_INSIDE is
 * the caller's guarantee that every particle's cell lies in [clo, chi) on entry (the wrap keeps
 * them there).  With it, when no node clo-1 .. chi is in a PML column, the streaming path may
 * carry each step's H phase in the next step's push launch (the push then forms H^(t+1/2) at its
 * nodes itself), taking one dependent launch out of each step; same results. */
#define FDTDPIC_PATH_MODE 15
#define FDTDPIC_PATH_CELLS_INSIDE 16

typedef struct PicBeam {
    int32_t n_part;     /* macroparticles */
    int32_t clo, chi;   /* periodic beam domain, cells [clo, chi); 2 <= clo < chi <= nz-2 */
    int32_t sort_every; /* re-bin by cell every this many steps (0: never) */
    int32_t chunk;      /* particles per CTA in the push kernel (0: library default) */
    int32_t path;       /* 0: automatic (= streaming, measured faster on GB300 at every size
                           but the smallest, where the two tie), 1: streaming kernels,
                           2: persistent tiled kernel, 3: temporally blocked passes (long
                           grids: sort_every whole steps per launch, 0 for 8, over tiles of
                           about chunk cells, 0 for 512, each tile's fields and particles in
                           shared memory; FDTDPIC_ERR_ARG without
                           FDTDPIC_PATH_CELLS_INSIDE, for an empty beam, fewer than five
                           tiles, tiles narrower than twice the pass's halo H = 3 sort_every
                           + 4 cells, clo or chi within H cells of an edge of its tile (the
                           grid's ends excepted), the two tiles holding clo and chi within 2H
                           cells of each other, or a tile beyond shared memory); may be or-ed
                           with FDTDPIC_PATH_CELLS_INSIDE */
    double kE;     /* q dt / (2 m c) */
    double kH;     /* -q mu0 dt / (2 m) */
    double sc;     /* c dt / dz */
    double kJ;     /* q w c: Jx per unit ux/gamma */
    double kJz;    /* q w dz / dt: Jz per unit cell displacement */
    double jscale; /* deposit fixed-point scale, a power of two; see fdtdpic_pic_jscale */
} PicBeam;

/* Optional per-kernel GPU time of one fdtdpic_run call, from CUDA events recorded around every
 * launch (milliseconds summed over the call).  Passing a timing struct makes the call
 * synchronous and launches kernel by kernel instead of replaying captured graphs. */
typedef struct FdtdPicTiming {
    float push_ms;  /* gather + Boris push + deposit (with the previous step's H phase when
                       the push launch carries it, FDTDPIC_PATH_CELLS_INSIDE) */
    float field_ms; /* field step (E and H phases; E only where the push carries H) */
    float sort_ms;  /* re-binning by cell */
    int32_t steps;
    int32_t path;   /* 1: streaming kernels, 2: persistent tiled kernel (push_ms = whole kernel),
                       3: streaming kernels, each push launch carrying the previous H phase,
                       4: temporally blocked passes (push_ms = all passes) */
} FdtdPicTiming;

/* Bytes of caller scratch fdtdpic_run needs (deposit accumulators, re-binning buffers). */
int64_t fdtdpic_scratch_bytes(int precision, int nz, int n_part);
/* Bytes of scratch fdtdpic_run needs for this run on the current device: for beam->path == 2
 * the persistent tiled path's requirement (the tiled path applies when the grid splits into at
 * least two tiles of >= max(pml+2, 8) cells, one per SM, each fitting shared memory); for
 * path 3 (with FDTDPIC_PATH_CELLS_INSIDE) the temporally blocked path's (its particle segments,
 * double buffered, and a second copy of the state and of Hyp); else the streaming path's. */
int64_t fdtdpic_pic_scratch_bytes(int precision, const FdtdInstance *inst, const PicBeam *beam);
/* The largest power-of-two scale for which no deposit accumulator can overflow. */
double fdtdpic_pic_jscale(const PicBeam *beam);
/* The tiling a temporally blocked run (PicBeam.path mode 3) takes on a device with smem_optin
 * bytes of opt-in shared memory per CTA (cudaDevAttrMaxSharedMemoryPerBlockOptin; 232,448 on
 * GB300), computed on the host for beam->sort_every and beam->chunk whatever beam->path holds.
 * out (nullable, up to n_out values, in this order): steps a pass S, halo H = 3S+4 cells,
 * tiles G, narrowest and widest tile, a tile's loaded range wmax + 2H, the particles one loaded
 * range holds, shared memory of a one-tile CTA and of the CTA holding both wrap tiles, and
 * fdtdpic_run's scratch bytes.  Returns the number of values (10) when the path applies, else
 * FDTDPIC_ERR_ARG (the conditions at PicBeam.path). */
int fdtdpic_pass_plan(int precision, const FdtdInstance *inst, const PicBeam *beam,
                      int64_t smem_optin, int64_t *out, int n_out);

/* Steps [step_begin, step_end) of one instance coupled to a beam.  Fields live in d_state (as
 * fdtd1d_run_global); d_hyp (nz+1) holds Hy one half step back (zero for a fresh run) and is
 * updated.  Particle arrays (n_part each, T = precision's type): d_cell int32, d_frac, d_ux,
 * d_uz T, d_id int32 (an identity carried through re-binning); updated in place (re-binning
 * permutes them within each cell).  d_jx/d_jz (nz+1, T) receive the last step's grid currents.
 * d_status[0] += particles that left the grid, d_status[1] |= FDTD_STATUS_NONFINITE.
 * Blocks of 2*sort_every steps (64 without re-binning) are captured once into a CUDA graph and
 * replayed (the step index lives in the scratch), so a repeated call with the same arguments
 * reuses the graph; timing (nullable) is described at FdtdPicTiming. */
int fdtdpic_run(int precision, const FdtdInstance *h_inst, const FdtdInstance *d_inst,
                const double *d_pml_tab, const double *d_src, void *d_state, void *d_probe,
                const PicBeam *beam, int32_t *d_cell, void *d_frac, void *d_ux, void *d_uz,
                int32_t *d_id, void *d_jx, void *d_jz, void *d_hyp, void *d_scratch,
                int64_t scratch_bytes, int32_t *d_status, FdtdPicTiming *timing,
                fdtdpic_stream_t stream);

/* fdtdpic_run for callers that cannot allocate device memory (no counterpart in the
 * reference; the reference allocates nothing on a device).  For example code running inside
 * another framework's memory pool, or a plug-in in a host that has reserved the whole device.
 * Same arguments minus the scratch: it uses a 24 MiB array compiled into the library, held on
 * every device that loads the library until exit.  Runs needing more scratch than that
 * (fdtdpic_scratch_bytes > 24 MiB) return FDTDPIC_ERR_OOM.  All calls share the array, so calls
 * that overlap on the GPU race: serialise them.  The first call on a device looks up the array's
 * address (make it before any stream capture) and keeps it for the device's context: do not call
 * this entry point on a device after cudaDeviceReset.  Streaming kernels only: beam->path takes
 * the bits fdtdpic_run takes with mode 0 or 1 (modes 2 and 3, the tiled and pass paths, return
 * FDTDPIC_ERR_ARG).  Launches kernel by kernel; no cudaMalloc, no graph capture, no event or
 * stream creation. */
int fdtdpic_run_noalloc(int precision, const FdtdInstance *h_inst, const FdtdInstance *d_inst,
                        const double *d_pml_tab, const double *d_src, void *d_state, void *d_probe,
                        const PicBeam *beam, int32_t *d_cell, void *d_frac, void *d_ux,
                        void *d_uz, int32_t *d_id, void *d_jx, void *d_jz, void *d_hyp,
                        int32_t *d_status, fdtdpic_stream_t stream);

/* ---- served requests: continuous batching over slots ---------------------------------------
 * No counterpart in the reference, which runs one simulation per script invocation
 * (MasterController.LoopedSim, MasterController.py:530-600, loops over runs one at a time).
 * A slot is one admitted request with its own device buffers; a work item is a chunk of its
 * steps.  fdtdpic_slots_run runs a list of work items in one launch: each CTA takes the next
 * item from d_queue and steps that request's chunk alone, its fields in shared memory when they
 * fit (otherwise in the slot's global buffers), its beam (if any) pushed by the same CTA with
 * exact fixed-point deposits.  A request's results therefore depend only on its own inputs and
 * its chunk boundaries, never on which other requests share the launch.  Between launches the
 * caller admits new requests into free slots and retires finished ones. */
typedef struct FdtdSlot {
    FdtdInstance inst;     /* offsets are into this slot's buffers below; step_begin, step_end
                              and resume are taken from the work item */
    const double *pml_tab; /* FDTD_TAB_ROWS x (2 pml + 1) */
    const double *src;     /* Exs[n_steps] then Hys[n_steps] */
    void *state;           /* FDTD_STATE_ARRAYS x (nz+1), precision's type */
    void *probe;           /* [n_steps][2] */
    void *hist;            /* [hist_rows][nz+1] or NULL */
    int32_t n_part;        /* 0: a field-only request; the beam fields below are then unused */
    int32_t clo, chi;      /* periodic beam domain [clo, chi), 2 <= clo < chi <= nz-2 */
    int32_t reserved;
    int32_t *cell;         /* n_part particles: cell, frac, ux, uz as for fdtdpic_run */
    void *frac, *ux, *uz;
    void *hyp;             /* (nz+1): Hy one half step back */
    void *jx, *jz;         /* (nz+1): the last step's grid currents */
    uint64_t *acc;         /* 2 x words x (nz+1) deposit accumulators (words: 1 for FDTDPIC_F32,
                              2 for FDTDPIC_F64), used when they do not fit shared memory */
    double kE, kH, sc, kJ, kJz, jscale; /* as PicBeam */
    int32_t status[4];     /* written by the kernel: [0] += particles outside the grid,
                              [1] |= FDTD_STATUS_* bits, [2] += FP64 cubic re-solves */
} FdtdSlot;

typedef struct FdtdSlotItem {
    int32_t slot;  /* index into the slot array */
    int32_t t0;    /* steps [t0, t1) of that request */
    int32_t t1;
    int32_t first; /* 1: t0 starts the request (zero fields, zero beam history) */
} FdtdSlotItem;

/* ---- set-up on the device -------------------------------------------------------------------
 * The per-grid set-up of the reference, for a whole ragged batch in one launch: the CPML
 * profile and coefficient arrays of boundCondManager (Solver_Engine.py:70-87: CPML_ScalingCalc,
 * CPML_Ex_RC_Define, CPML_HY_RC_Define, CPML_Ex_Update_Coef, CPML_Hy_Update_Coef and
 * denominators, BaseFDTD11.py:223-357) as the instance's PML table; UpExMat/UpHyMat
 * (EmptySpaceCalc / Material + UpdateCoef, BaseFDTD11.py:124-132); the Kerr cubic's
 * coefficients (Nonlin_Eqn_Setup / AcubicFinder, :795-820) and the Lorentz ADE's A, B, C
 * (ADE_TempPolCurr, :487-538).  The plasma frequency comes in already corrected by
 * genericStability.spatialStab (genericStability.py:12-62). */
typedef struct FdtdSetup {
    double dz, dt;        /* Params.dz, Params.delT */
    double courant;       /* Params.courantNo (the float32 value) */
    double eps0, mu0;     /* permit_0, permea_0 */
    double char_imp;      /* Params.CharImp */
    double eps_re, mu_re; /* slab epsRe, muRe (free-space integrator) */
    double kappa_max, sigma_opt, alpha_max, r_scale, r_a_scale; /* CPML_Params */
    double plasma_freq;   /* Variables.plasmaFreqE after spatialStab */
    double omega0, gamma; /* omega_0E, gammaE */
    double chi3, alpha3;  /* chi3Stat, alpha3 */
    double freq_in;       /* Params.freq_in */
    int32_t free_space;   /* 1: the slab takes UpExMat/epsRe, UpHyMat/muRe */
    int32_t reserved;
} FdtdSetup;

/* For each instance i: reads its geometry (nz, pml, cpml_lo, cpml_hi, pml_offset) from
 * d_inst[i], writes its coefficient fields (ue, ue_slab, uh, uh_slab, dtdz, eps0, sc, pol_a..c,
 * kerr_a..c, nl_e0, nl_e0chi) and its FDTD_TAB_ROWS x (2 pml + 1) table at
 * d_pml_tab + pml_offset.  All arrays in device memory; asynchronous on the stream. */
int fdtdpic_setup_batch(int n_inst, const FdtdSetup *d_setup, FdtdInstance *d_inst,
                        double *d_pml_tab, fdtdpic_stream_t stream);
/* Like fdtdpic_instance_layout, for FdtdSetup. */
int fdtdpic_setup_layout(int64_t *out, int n);

/* Like fdtdpic_instance_layout, for FdtdSlot. */
int fdtdpic_slot_layout(int64_t *out, int n);
/* Host-side check of one slot descriptor before it is admitted (FDTDPIC_OK or ERR_ARG). */
int fdtdpic_slot_check(int precision, const FdtdSlot *slot);
/* Shared memory (bytes) with which this slot's fields (field-only request) or deposit
 * accumulators (beam request) stay on chip; host-only. */
int64_t fdtdpic_slot_smem_bytes(int precision, const FdtdSlot *slot);
/* CTAs one fdtdpic_slots_run launch keeps resident with these settings (grid_ctas <= 0 picks
 * this many); 0 when the settings are invalid or no device is usable. */
int fdtdpic_slots_grid(int precision, int64_t smem_bytes, int threads_per_cta);
/* Run n_items work items over n_slots slots (both arrays in device memory) in one launch.
 * d_queue: one int32 of caller scratch, reset by this call.  smem_bytes: dynamic shared memory
 * per CTA (items whose slot needs more run from global memory).  threads_per_cta <= 0 picks
 * 512; grid_ctas <= 0 the occupancy-limited grid.  Items naming a slot outside [0, n_slots) or
 * a step range outside [0, n_steps] are skipped and flagged in the slot's status[1]
 * (FDTD_STATUS_SKIPPED) when the slot exists. */
int fdtdpic_slots_run(int precision, FdtdSlot *d_slots, int n_slots, const FdtdSlotItem *d_items,
                      int n_items, int32_t *d_queue, int64_t smem_bytes, int threads_per_cta,
                      int grid_ctas, fdtdpic_stream_t stream);

/* ---- Per-step variants the reference defines but never calls (its call sites are commented
 * out or absent): the first-order Mur edge update, the JEC polarisation current and Varin's
 * explicit nonlinear Lorentz/Kerr/Raman ADE.  Each operation updates rows of device arrays
 * (row r at element r * stride, the row's first n elements) with the reference function's
 * arithmetic, in its operation order (FP64: the same values; FP32: float arrays and float
 * arithmetic on coefficients formed in FP64).
 *
 *   FDTD_VAR_MUR_EX    MUR1DEx (BaseFDTD11.py:769-788; call sites Solver_Engine.py:187,318,321)
 *                      a0 = Ex (in/out), a1 = tempTempVarE.  m = (c0 dt - dz)/(c0 dt + dz);
 *                      Ex[k] = E2[k+1] + m (Ex[k+1] - E2[k]) for k = 1..4, then
 *                      Ex[k] = E2[k-1] + m (Ex[k-1] - E2[k]) for k = Nz-1 down to Nz-5, each
 *                      reading Ex as the reference's loops leave it.  Needs 6 <= nz <= n.
 *   FDTD_VAR_ADE_JX    ADE_JxUpdate (:543-563; call sites Solver_Engine.py:244,302)
 *                      a0 = Jx (out), a1 = polarisationCurr, a2 = tempVarPol,
 *                      a3 = tempTempVarPol; cells front-1 .. rear-1;
 *                      Jx = c (w0E^2 P1 + (gammaE/dt)(P - P1) + (P - 2 P1 + P2)/dt^2),
 *                      c = 1/(eps0 wp w0E w0j).  Needs 1 <= front, rear <= n.
 *   FDTD_VAR_VARIN_PBAR ADE_NonLin_Pol_Ex_Pbar (:567-576)
 *                      a0 = Pbar3 (out), a1 = Ex, a2 = Qx3; cells front .. rear-1;
 *                      Pbar3 = eps0 (chi1 E + chi3 (alpha3 E^3 + (1 - alpha3) Q E)).
 *   FDTD_VAR_VARIN_JP  ADE_Lin_Curr_And_Pol_Varin (:579-593)
 *                      a0 = Jx (in/out), a1 = polarisationCurr (in/out), a2 = Pbar3;
 *                      J = (A/D) J + (B/D)(Pbar3 - P), then P = P + dt J, with
 *                      G = gammaE dt/2, A = 1 - G, D = 1 + G, B = w0E^2 dt.
 *   FDTD_VAR_VARIN_QG  ADE_Nonlin_Q_and_G (:596-607)
 *                      a0 = Gx3 (in/out), a1 = Qx3 (in/out), a2 = Ex;
 *                      G = (e/f) G + (h/f)(E^2 - Q), then Q = Q + dt G, with
 *                      g = nonLin3gammaE dt/2, e = 1 - g, f = 1 + g, h = nonLin3Omega_0E^2 dt.
 *   FDTD_VAR_VARIN_STEP the three Varin updates of one cell in one pass (PBAR, JP, QG in that
 *                      order; the same values as the three calls): a0 = Pbar3, a1 = Jx,
 *                      a2 = polarisationCurr, a3 = Gx3, a4 = Qx3, a5 = Ex.
 * The Varin ranges need 0 <= front, rear <= n; front >= rear is an empty range. */
#define FDTD_VAR_MUR_EX 0
#define FDTD_VAR_ADE_JX 1
#define FDTD_VAR_VARIN_PBAR 2
#define FDTD_VAR_VARIN_JP 3
#define FDTD_VAR_VARIN_QG 4
#define FDTD_VAR_VARIN_STEP 5

typedef struct FdtdVariantRow {
    int32_t n;              /* elements of this row's arrays */
    int32_t nz;             /* Params.Nz (MUR1DEx's right edge) */
    int32_t front, rear;    /* Params.materialFrontEdge, materialRearEdge */
    double c0, dt, dz;      /* Params.c0, delT, dz */
    double eps0;            /* Params.permit_0 */
    double plasma_freq;     /* Variables.plasmaFreqE */
    double omega0, gamma;   /* Variables.omega_0E, gammaE */
    double omega0_j;        /* Variables.omega_0 (read by ADE_JxUpdate only) */
    double chi1, chi3;      /* Variables.chi1Stat, chi3Stat */
    double alpha3;          /* Variables.alpha3 (the float32 value) */
    double nl_gamma;        /* Variables.nonLin3gammaE */
    double nl_omega0;       /* Variables.nonLin3Omega_0E */
} FdtdVariantRow;

/* Like fdtdpic_instance_layout, for FdtdVariantRow. */
int fdtdpic_variant_layout(int64_t *out, int n);
/* Host-side check of rows for an operation (FDTDPIC_OK or FDTDPIC_ERR_ARG). */
int fdtdpic_variant_check(int op, int n_rows, const FdtdVariantRow *h_rows, int64_t stride);
/* Apply operation `op` to n_rows rows.  h_rows (host) is checked as fdtdpic_variant_check does;
 * d_rows is its device copy, which the kernel reads.  arrays: the operation's device arrays
 * a0, a1, ... in the order above (FDTDPIC_F32: float, FDTDPIC_F64: double), each holding
 * n_rows rows of `stride` elements.  Asynchronous on the stream. */
int fdtdpic_variant_run(int op, int precision, int n_rows, const FdtdVariantRow *h_rows,
                        const FdtdVariantRow *d_rows, int64_t stride, void *const *arrays,
                        fdtdpic_stream_t stream);

/* ---- Bounded waits ----------------------------------------------------------------------
 * The persistent tiled PIC kernel's waits on its neighbours give up at a per-run deadline
 * (default 20 s plus 1 ms per step) and the tensor-core DFT's mbarrier waits after a poll
 * limit; a wait that gives up reports FDTDPIC_ERR_TIMEOUT (the tiled run's status word gets
 * FDTD_STATUS_TIMEOUT, the DFT's d_err is set) and its kernel returns, so the context stays
 * usable.  No counterpart in the reference, whose only failure handling is print + sys.exit
 * (Environment_Setup.py:59-155) and breakpoint() (BaseFDTD11.py:535-537). */
/* Set the tiled kernel's per-run deadline in nanoseconds for the runs launched after this call
 * (0: the default).  Process-wide; meant for tests that make a run's waits run out (a wait
 * that starts after the deadline gives up at once). */
int fdtdpic_set_run_deadline(int64_t ns);
/* One thread waits on something nothing completes and must give up.  which = 0: the tiled
 * kernel's neighbour-flag wait on a flag nothing raises, deadline `limit` ns (<= 2e9) from its
 * start (d_scratch: 2 int32 of device scratch, the flag and the abort word); which = 1: the
 * DFT's mbarrier wait on a barrier nothing arrives on, `limit` polls (<= 2^26; d_scratch
 * unused).  d_out (2 int32, device): [0] the code the wait reported (FDTDPIC_ERR_TIMEOUT when it
 * gave up), [1] microseconds it waited. */
int fdtdpic_wait_selftest(int which, int64_t limit, int32_t *d_out, int32_t *d_scratch,
                          fdtdpic_stream_t stream);

/* ---- Per-step updates, one launch each ----------------------------------------------------
 * The unit of work of the reference's module functions, for callers that build their own time
 * loop from them.  Each operation updates cells [lo, hi) of FP64 device arrays (n elements
 * each; arrays[i] is slot a<i>, NULL where the operation allows it) with the reference's
 * arithmetic in its operation order.  Cells of a range are independent (a cell writes only its
 * own elements and reads neighbours of arrays the operation does not write).
 *
 *   FDTD_OP_CURL       a0 = y (in/out), a1 = x, a2 = s (NULL: 1), a3 = j (NULL: 0),
 *                      a4..a6 = factor arrays (NULL: the scalar fval[i]):
 *                      y[k] = y[k]*s[k] + ((x[k+xa] - x[k+xb]) - j[k]) op0 f0 op1 f1 op2 f2,
 *                      op_i by fmode[i]: 0 skip, 1 multiply, 2 divide (left to right).
 *                      BaseFDTD11.ADE_ExUpdate (BaseFDTD11.py:664), ADE_HyUpdate (:641),
 *                      ADE_DxUpdate (:751); BaseFDTD.ADE_ExUpdate (BaseFDTD.py:401),
 *                      ADE_HyUpdate (:392), CPML_ExUpdate (:357), CPML_HyUpdate (:351),
 *                      ADE_DxUpdate (:418, its Dx half).
 *   FDTD_OP_PSI        a0 = psi (in/out), a1 = y (in/out), a2 = x, a3 = b, a4 = c, a5 = C:
 *                      psi = b*psi + c*(x[k+xa] - x[k+xb]); y = y + C*psi (s[0] >= 0) or
 *                      y - C*psi (s[0] < 0).  BaseFDTD11.CPML_Psi_e_Update (:365),
 *                      CPML_Psi_m_Update (:382); BaseFDTD.CPML_Psi_e_Update (:334),
 *                      CPML_Psi_m_Update (:342).
 *   FDTD_OP_POL        a0 = y (out), a1 = p1, a2 = p2, a3 = x: y = (A p1 + B p2) + C x with
 *                      s = (A, B, C).  BaseFDTD11.ADE_PolarisationCurrent_Ex (:610, p1 = y),
 *                      BaseFDTD.ADE_PolarisationCurrent_Ex (:378, p1 = tempVarPol).
 *   FDTD_OP_EXCREATE   a0 = y (out), a1 = u, a2 = v: y = (u - v) / s[0].  ADE_ExCreate
 *                      (BaseFDTD11.py:713, BaseFDTD.py:413), BaseFDTD.ADE_DxUpdate's Ex half.
 *   FDTD_OP_NONLIN_EX  a0 = y (out), a1 = Dx, a2 = Acubic: y = Dx / (s[0] + s[1] Acubic) with
 *                      s = (permit_0 Re(sqrt(1.2)), permit_0 chi3Stat).  NonLinExUpdate (:859).
 *   FDTD_OP_ACUBIC     a0 = Acubic (out), a1 = Dx, a2 = d (out; NULL: not written):
 *                      d = -|Dx/s[0]|^2, Acubic = Re(CubicEquationSolver.solve(s[1], s[2],
 *                      s[3], d)[0]) when |d| > 1e-8, else 0.  AcubicFinder (:803) with
 *                      Nonlin_Eqn_Setup (:795) and Nonlin_Cubic_Solver (:824); s = (permit_0,
 *                      cub, qua, one).
 * Stencil offsets xa, xb lie in {-1, 0, 1}; every stencil read must stay inside [0, n). */
#define FDTD_OP_CURL 0
#define FDTD_OP_PSI 1
#define FDTD_OP_POL 2
#define FDTD_OP_EXCREATE 3
#define FDTD_OP_NONLIN_EX 4
#define FDTD_OP_ACUBIC 5
#define FDTD_STEP_OP_ARRAYS 8

typedef struct FdtdStepOp {
    int32_t op;       /* FDTD_OP_* */
    int32_t lo, hi;   /* cells [lo, hi) */
    int32_t xa, xb;   /* stencil offsets (CURL, PSI) */
    int32_t fmode[3]; /* CURL factors: 0 skip, 1 multiply, 2 divide */
    double fval[3];   /* CURL scalar factors (used where the factor array is NULL) */
    double s[4];      /* the operation's scalars */
} FdtdStepOp;

/* Like fdtdpic_instance_layout, for FdtdStepOp. */
int fdtdpic_step_op_layout(int64_t *out, int n);
/* Host-side check of an operation and its array slots (FDTDPIC_OK or FDTDPIC_ERR_ARG). */
int fdtdpic_step_op_check(const FdtdStepOp *op, double *const *arrays, int64_t n);
/* Run one operation (arrays: FDTD_STEP_OP_ARRAYS device pointers, a host array); asynchronous
 * on the stream. */
int fdtdpic_step_op(const FdtdStepOp *op, double *const *arrays, int64_t n,
                    fdtdpic_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* FDTDPIC_H */
