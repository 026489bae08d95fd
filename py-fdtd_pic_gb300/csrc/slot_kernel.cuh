// Served requests: one launch runs a list of work items (a request's chunk of steps); each CTA
// takes items from a device queue and steps each one alone.
//
//   field-only request, fields fit shared memory : run_instance_resident (the batch kernel's
//                                                   per-instance loop)
//   field-only request, larger                   : run_instance_cta_global (same step, fields in
//                                                   the slot's global buffers, L2-resident)
//   request with a beam                          : run_beam_slot (push, deposit, field step per
//                                                   step; fields global, deposit accumulators in
//                                                   shared memory when they fit)
//
// A beam request's step is the streaming PIC path's step (pic_kernel.cuh) operation for
// operation: the same particle_step, the same exact int64 deposits (so particle order does not
// matter), the same E phase (Hyp <- Hy, currents out of the accumulators, e_cell with -Jx) and H
// phase; built with the same flags (-fmad=false) its results equal fdtdpic_run's bit for bit.
#pragma once
#include "fdtd1d_kernel.cuh"
#include "pic_kernel.cuh"

namespace fdtdpic {

struct SlotArgs {
    FdtdSlot *slots;
    int n_slots;
    const FdtdSlotItem *items;
    int n_items;
    int32_t *queue;
    int64_t smem_bytes;
};

template <typename T>
__device__ inline BatchArgs<T> slot_batch_args(FdtdSlot &S)
{
    BatchArgs<T> a{1, nullptr, nullptr, S.pml_tab, S.src, (T *)S.state, (T *)S.probe,
                   (T *)S.hist, nullptr, &S.status[1], &S.status[2], 0};
    return a;
}

// Field-only request of any size in one CTA, fields in global memory.
template <typename T>
__device__ void run_instance_cta_global(const BatchArgs<T> &args, const FdtdInstance &I)
{
    const int tid = threadIdx.x, nt = blockDim.x;
    const int n = I.nz + 1;
    GlobalStore<T> s = global_store<T>(I, args);
    T *gst = args.state + I.state_offset;
    T *gA = gst + (int64_t)FDTD_ST_A * n;
    if (!I.resume)
        for (int64_t i = tid; i < (int64_t)FDTD_STATE_ARRAYS * n; i += nt) gst[i] = T(0);
    __shared__ T s_src[2][2];
    __syncthreads();
    if (tid == 0 && I.step_begin < I.step_end) {
        s_src[I.step_begin & 1][0] = src_e_at<T>(I, args.src, I.step_begin);
        s_src[I.step_begin & 1][1] = src_h_at<T>(I, args.src, I.step_begin);
    }
    __syncthreads();
    const Scal<T> c = make_scal<T>(I);
    Kerr<T> kr;
    kr.setup(I);
    T *probe = args.probe + I.probe_offset;
    T *hist = args.hist ? args.hist + I.hist_offset : nullptr;
    int nfb = 0;
    for (int t = I.step_begin; t < I.step_end; ++t) {
        const T src_e = s_src[t & 1][0];
        const T src_h = s_src[t & 1][1];
        T *a_out = (t == I.step_end - 1) ? gA : nullptr;
        for (int k = 1 + tid; k < n; k += nt)
            e_cell<T>(I, c, kr, s, k, src_e, src_h, false, T(0), a_out, &nfb);
        __syncthreads();
        for (int k = 1 + tid; k < n - 1; k += nt) h_cell<T>(I, c, s, k, src_h);
        if (tid == 0) tfsf_edge<T>(I, s, src_h);
        // probes and snapshots read Ex, which the H phase does not write
        if (tid < 2 && t >= I.probe_lo[tid] && t <= I.probe_hi[tid])
            probe[(int64_t)t * 2 + tid] = s.Ex(I.probe_cell[tid]);
        if (hist && I.hist_interval > 0 && t > 0 && (t % I.hist_interval) == 0) {
            const int row = t / I.hist_interval;
            if (row < I.hist_rows)
                for (int k = tid; k < n; k += nt) hist[(int64_t)row * n + k] = s.Ex(k);
        }
        if (tid == nt - 1 && t + 1 < I.step_end) {
            s_src[(t + 1) & 1][0] = src_e_at<T>(I, args.src, t + 1);
            s_src[(t + 1) & 1][1] = src_h_at<T>(I, args.src, t + 1);
        }
        __syncthreads();
    }
    bool bad = false;
    for (int k = tid; k < n; k += nt) bad |= !(isfinite((double)s.Ex(k)) && isfinite((double)s.Hy(k)));
    if (bad && args.status) atomicOr(args.status, FDTD_STATUS_NONFINITE);
    if (nfb && args.fallbacks) atomicAdd(args.fallbacks, nfb);
}

// Add one particle's deposit words to the accumulators (shared: exact 32-bit pairs; global:
// native 64-bit atomics).
template <int W>
__device__ __forceinline__ void slot_deposit(unsigned long long *acc, bool shared, int n,
                                             int word0, int node, const long long *v)
{
#pragma unroll
    for (int w = 0; w < W; ++w) {
        const unsigned long long u = (unsigned long long)v[w];
        if (u == 0ull) continue;
        unsigned long long *p = acc + (size_t)(word0 + w) * n + node;
        if (shared)
            smem_add_u64(p, u);
        else
            atomicAdd(p, u);
    }
}

template <typename T>
__device__ void run_beam_slot(FdtdSlot &S, const FdtdInstance &I, unsigned char *smem_raw,
                              int64_t smem_bytes)
{
    constexpr int W = Fix<T>::W;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int n = I.nz + 1;
    BatchArgs<T> fa = slot_batch_args<T>(S);
    GlobalStore<T> s = global_store<T>(I, fa);
    T *gst = fa.state + I.state_offset;
    T *gA = gst + (int64_t)FDTD_ST_A * n;
    T *hyp = (T *)S.hyp, *jx = (T *)S.jx, *jz = (T *)S.jz;
    int32_t *cell = S.cell;
    T *frac = (T *)S.frac, *ux = (T *)S.ux, *uz = (T *)S.uz;
    const int64_t acc_words = 2 * (int64_t)W * n;
    const bool acc_shared = acc_words * 8 <= smem_bytes;
    unsigned long long *acc =
        acc_shared ? reinterpret_cast<unsigned long long *>(smem_raw) : (unsigned long long *)S.acc;
    if (!I.resume) {
        for (int64_t i = tid; i < (int64_t)FDTD_STATE_ARRAYS * n; i += nt) gst[i] = T(0);
        for (int k = tid; k < n; k += nt) hyp[k] = T(0);
    }
    // accumulators are zero between steps; shared ones start each chunk zeroed, global ones
    // are zeroed with the fresh fields
    if (acc_shared || !I.resume)
        for (int64_t i = tid; i < acc_words; i += nt) acc[i] = 0ull;
    const T kE = (T)S.kE, kH = (T)S.kH, scb = (T)S.sc, kJ = (T)S.kJ, kJz = (T)S.kJz;
    const double jscale = S.jscale, jinv = 1.0 / S.jscale;
    const float jscale_f = (float)S.jscale, jinv_f = (float)(1.0 / S.jscale);
    const int np = S.n_part, clo = S.clo, chi = S.chi, Lc = chi - clo;
    const Scal<T> c = make_scal<T>(I);
    Kerr<T> kr;
    kr.setup(I);
    T *probe = fa.probe + I.probe_offset;
    T *hist = fa.hist ? fa.hist + I.hist_offset : nullptr;
    __shared__ T s_src[2];
    int nfb = 0, lost = 0;
    __syncthreads();
    for (int t = I.step_begin; t < I.step_end; ++t) {
        const bool last = (t == I.step_end - 1);
        if (tid == 0) {
            s_src[0] = src_e_at<T>(I, fa.src, t);
            s_src[1] = src_h_at<T>(I, fa.src, t);
        }
        // push: gather E^t and B^t, Boris, move, deposit Jx^(t+1/2) (and Jz on the last step)
        for (int p = tid; p < np; p += nt) {
            const int cp = cell[p];
            const T f = frac[p];
            if (cp < 1 || cp + 2 > I.nz) { ++lost; continue; }
            int j;
            T fh;
            if (f >= T(0.5)) { j = cp; fh = f - T(0.5); } else { j = cp - 1; fh = f + T(0.5); }
            const T E = (T(1) - f) * s.Ex(cp) + f * s.Ex(cp + 1);
            const T H = (T(1) - fh) * (T(0.5) * (s.Hy(j) + hyp[j])) +
                        fh * (T(0.5) * (s.Hy(j + 1) + hyp[j + 1]));
            Moved<T> m;
            particle_step<T>(E, H, cp, f, ux[p], uz[p], kE, kH, scb, kJ, m);
            long long v[W];
            Fix<T>::split(m.jx0, jscale, jscale_f, v);
            slot_deposit<W>(acc, acc_shared, n, 0, m.nx0, v);
            Fix<T>::split(m.jx1, jscale, jscale_f, v);
            slot_deposit<W>(acc, acc_shared, n, 0, m.nx0 + 1, v);
            if (last) {
                const MovedJz<T> z = particle_jz<T>(cp, f, m, kJz);
                Fix<T>::split(z.jzA, jscale, jscale_f, v);
                slot_deposit<W>(acc, acc_shared, n, W, z.nzA, v);
                if (z.nzB >= 0) {
                    Fix<T>::split(z.jzB, jscale, jscale_f, v);
                    slot_deposit<W>(acc, acc_shared, n, W, z.nzB, v);
                }
            }
            int c1 = m.c1;
            if (c1 >= chi) c1 -= Lc;
            else if (c1 < clo) c1 += Lc;
            cell[p] = c1;
            frac[p] = m.f1;
            ux[p] = m.ux;
            uz[p] = m.uz;
        }
        __syncthreads();
        const T src_e = s_src[0], src_h = s_src[1];
        // E phase: Hyp <- Hy, currents out of the accumulators (zeroed), E update with -Jx
        for (int k = tid; k < n; k += nt) {
            hyp[k] = s.Hy(k);
            unsigned long long wx[W], wz[W];
#pragma unroll
            for (int w = 0; w < W; ++w) {
                wx[w] = acc[(size_t)w * n + k];
                wz[w] = acc[(size_t)(W + w) * n + k];
                acc[(size_t)w * n + k] = 0ull;
                acc[(size_t)(W + w) * n + k] = 0ull;
            }
            const T jxk = Fix<T>::join(wx, jinv, jinv_f);
            jx[k] = jxk;
            jz[k] = Fix<T>::join(wz, jinv, jinv_f);
            if (k >= 1) e_cell<T>(I, c, kr, s, k, src_e, src_h, true, jxk, gA, &nfb, true);
        }
        __syncthreads();
        for (int k = 1 + tid; k < n - 1; k += nt) h_cell<T>(I, c, s, k, src_h);
        if (tid == 0) tfsf_edge<T>(I, s, src_h);
        if (tid < 2 && t >= I.probe_lo[tid] && t <= I.probe_hi[tid])
            probe[(int64_t)t * 2 + tid] = s.Ex(I.probe_cell[tid]);
        if (hist && I.hist_interval > 0 && t > 0 && (t % I.hist_interval) == 0) {
            const int row = t / I.hist_interval;
            if (row < I.hist_rows)
                for (int k = tid; k < n; k += nt) hist[(int64_t)row * n + k] = s.Ex(k);
        }
        __syncthreads();
    }
    bool bad = false;
    for (int k = tid; k < n; k += nt) bad |= !(isfinite((double)s.Ex(k)) && isfinite((double)s.Hy(k)));
    if (bad) atomicOr(&S.status[1], FDTD_STATUS_NONFINITE);
    if (lost) atomicAdd(&S.status[0], lost);
    if (nfb) atomicAdd(&S.status[2], nfb);
}

template <typename T>
__global__ void __launch_bounds__(1024) fdtdpic_slot_kernel(SlotArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int next;
    while (true) {
        if (threadIdx.x == 0) next = atomicAdd(a.queue, 1);
        __syncthreads();
        const int q = next;
        __syncthreads();
        if (q >= a.n_items) break;
        const FdtdSlotItem it = a.items[q];
        if (it.slot < 0 || it.slot >= a.n_slots) continue;
        FdtdSlot &S = a.slots[it.slot];
        __shared__ FdtdInstance s_inst;
        copy_instance_block(s_inst, S.inst);
        const FdtdInstance &I = s_inst;
        if (it.t0 < 0 || it.t1 < it.t0 || it.t1 > I.n_steps) {
            if (threadIdx.x == 0) atomicOr(&S.status[1], FDTD_STATUS_SKIPPED);
            continue;
        }
        if (threadIdx.x == 0) {
            s_inst.step_begin = it.t0;
            s_inst.step_end = it.t1;
            s_inst.resume = it.first ? 0 : 1;
        }
        __syncthreads();
        if (S.n_part > 0) {
            run_beam_slot<T>(S, I, smem_raw, a.smem_bytes);
        } else {
            const BatchArgs<T> fa = slot_batch_args<T>(S);
            if (resident_elems<T>(I) * (int64_t)sizeof(T) <= a.smem_bytes)
                run_instance_resident<T>(fa, I, 0, reinterpret_cast<T *>(smem_raw));
            else
                run_instance_cta_global<T>(fa, I);
        }
        __syncthreads();
    }
}

}  // namespace fdtdpic
