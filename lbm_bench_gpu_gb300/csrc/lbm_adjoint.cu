// lbm_adjoint.cu -- lbm_step_adjoint: gradient of a light-phase objective with
// respect to the body force and the initial phi field, by the discrete adjoint
// of the fused step with binomial checkpointing.  No counterpart in the
// reference.
//
// Schedule.  The forward trajectory s^0 .. s^T is not kept: native state
// snapshots (the step's own buffers, 26 distributions) go into a pool of slots
// sized from the memory budget, and missing states are recomputed from the
// nearest snapshot (Griewank's binomial checkpointing).  A segment [s, e) of
// length l with its start stored and c free slots has n = c + 1 snapshots;
// with r sweeps at most beta(n, r) = C(n + r, r) steps can be reversed, and
// the minimum of forward steps, r l - beta(n + 1, r - 1) for the smallest r
// with beta(n, r) >= l, is reached when the first checkpoint m lies in
//   [max(beta(n, r - 2), l - beta(n - 1, r)), min(beta(n, r - 1), l - beta(n - 1, r - 1))]
// steps from s (found by dynamic programming over the recursion below, and
// checked against the formula): m is stored, [m, e) is reversed with c - 1
// free slots, then [s, m) with c.  The lower end of the range is taken.
// Measured on the recursion: 20 000 steps with 44 slots take 62 709 forward
// steps (the minimum is 62 705), against 76 692 when m is placed so that the
// right part is as long as c - 1 slots allow.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "lbm_internal.h"

namespace {

using lbm::cuda_fail;
using lbm::fail;

double beta(int c, int r)
{
    // C(c + r, r), saturating
    double v = 1.0;
    for (int i = 1; i <= r; i++) {
        v = v * (double)(c + i) / (double)i;
        if (v > 1e18) return 1e18;
    }
    return v;
}

// Sub-buffers of one allocation, 256-byte aligned; with base == nullptr only
// the size is counted.
struct Carver {
    unsigned char *base;
    size_t off = 0;
    template <typename T>
    T *take(size_t count)
    {
        off = (off + 255) & ~(size_t)255;
        T *p = base ? reinterpret_cast<T *>(base + off) : nullptr;
        off += sizeof(T) * count;
        return p;
    }
};

// First checkpoint of a segment of len >= 2 steps with its start stored and
// cfree >= 1 free slots: the lower end of Griewank's optimal interval (see the
// file comment).
long long split_point(long long len, int cfree)
{
    const int n = cfree + 1;
    int r = 1;
    while (beta(n, r) < (double)len) r++;
    const double lo = std::max(r >= 2 ? beta(n, r - 2) : 1.0, (double)len - beta(n - 1, r));
    return std::max<long long>(1, std::min<long long>((long long)lo, len - 1));
}

// Forward steps of revolve(s, s + len, cfree) below, without running them
// (the same recursion; `terminal` is whether lambda^T is still to be built).
long long schedule_steps(long long T, long long s, long long e, int cfree, bool &terminal)
{
    const long long len = e - s;
    if (len <= 0) return 0;
    if (len == 1) {
        if (terminal) {
            terminal = false;
            return 1;
        }
        return 0;
    }
    if (cfree == 0) {
        long long steps = 0;
        for (long long j = e - 1; j >= s; j--) {
            if (terminal) {
                terminal = false;
                steps += T - s;
            }
            if (j != s) steps += j - s;
        }
        return steps;
    }
    const long long m = s + split_point(len, cfree);
    long long steps = m - s;
    steps += schedule_steps(T, m, e, cfree - 1, terminal);
    steps += schedule_steps(T, s, m, cfree, terminal);
    return steps;
}

struct Snapshot {
    long long step = -1;
    bool f_streamed = false, g_odd_next = false;
};

struct Adjoint {
    lbm_ctx *c;
    lbm_adjoint_opts o;
    size_t n, snap_bytes;
    // work buffers; phi and the objective sums ab (4 doubles) are
    // double-buffered by step parity so that the side stream can prepare
    // step n while the main stream still runs step n + 1
    float *phi = nullptr;     // 2 x n
    float *lam[2] = {nullptr, nullptr};   // 26 x n each: f (7) then g (19)
    float *lst[2] = {nullptr, nullptr};
    float4 *lsrc = nullptr;
    float *phi0 = nullptr, *mom_save = nullptr;
    double *partials = nullptr, *dgrav = nullptr, *ab = nullptr, *acc = nullptr;
    unsigned char *slots = nullptr;   // the context's checkpoint pool
    std::vector<Snapshot> snaps;
    unsigned char *host = nullptr;    // pinned host checkpoints (second tier), slot layout
    std::vector<Snapshot> hsnaps;
    std::vector<int> free_slots;
    int cur = 0;                 // lam[cur] holds lambda^{k+1}
    bool lambda_ready = false;
    long long fwd_steps = 0, adj_steps = 0;
    lbm::StepConst k;
    int first_source;            // first state index with an objective term
    double scale;
    // Side stream: phi and the objective of state n depend only on that
    // state, so they run there as soon as it exists, overlapping the main
    // stream's adjoint kernels of step n + 1.  Events order the two streams:
    // slot_ev[s] / ctx_ev mark a state written, buf_free[b] the main stream's
    // last read of phi / ab buffer b, side_done the side work of a step.
    cudaStream_t side = nullptr;
    std::vector<cudaEvent_t> slot_ev;
    cudaEvent_t ctx_ev = nullptr, side_done = nullptr, buf_free[2] = {nullptr, nullptr};

    float *phi_buf(long long step) { return phi + (size_t)(step & 1) * n; }
    double *ab_buf(long long step) { return ab + 4 * (step & 1); }

    int record(cudaEvent_t ev, cudaStream_t st)
    {
        if (!ev) return LBM_OK;
        cudaError_t e = cudaEventRecord(ev, st);
        return e == cudaSuccess ? LBM_OK : cuda_fail(e, "adjoint: event");
    }

    int create_streams(int nslots)
    {
        cudaError_t e = cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking);
        auto ev = [&](cudaEvent_t *p) {
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(p, cudaEventDisableTiming);
        };
        ev(&ctx_ev);
        ev(&side_done);
        ev(&buf_free[0]);
        ev(&buf_free[1]);
        slot_ev.assign((size_t)nslots, nullptr);
        for (auto &x : slot_ev) ev(&x);
        if (e == cudaSuccess) e = cudaEventRecord(buf_free[0], c->stream);
        if (e == cudaSuccess) e = cudaEventRecord(buf_free[1], c->stream);
        return e == cudaSuccess ? LBM_OK : cuda_fail(e, "adjoint: streams");
    }

    unsigned char *slot_ptr(int s) { return slots + (size_t)s * snap_bytes; }

    // the state in slot s, read in place
    lbm::NativeState slot_state(int s)
    {
        const unsigned char *d = slot_ptr(s);
        const size_t b0 = sizeof(float) * n, bq = c->esz * (lbm::kQf - 1) * n;
        return lbm::NativeState{c->p.storage, reinterpret_cast<const float *>(d), d + b0, d + b0 + bq,
                                snaps[s].f_streamed, snaps[s].g_odd_next};
    }

    // the context's current state
    lbm::NativeState ctx_state()
    {
        const lbm::StepView v = lbm::state_view(c, c->st.f_cur);
        return lbm::NativeState{c->p.storage, v.f0_in, v.fq_in, v.g, c->st.f_streamed, c->st.g_odd_next};
    }

    int save(int s, long long step)
    {
        lbm::StepView v = lbm::state_view(c, c->st.f_cur);
        unsigned char *d = slot_ptr(s);
        const size_t b0 = sizeof(float) * n, bq = c->esz * (lbm::kQf - 1) * n, bg = c->esz * lbm::kQg * n;
        cudaError_t e = cudaMemcpyAsync(d, v.f0_in, b0, cudaMemcpyDeviceToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d + b0, v.fq_in, bq, cudaMemcpyDeviceToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d + b0 + bq, c->st.g, bg, cudaMemcpyDeviceToDevice, c->stream);
        if (e != cudaSuccess) return cuda_fail(e, "adjoint: snapshot");
        snaps[s].step = step;
        snaps[s].f_streamed = c->st.f_streamed;
        snaps[s].g_odd_next = c->st.g_odd_next;
        return slot_ev.empty() ? LBM_OK : record(slot_ev[s], c->stream);
    }

    // the context's current state (at `step`) into host slot h, in the slot
    // layout; on the main stream, so the next step waits for the copy
    int to_host(int h, long long step)
    {
        lbm::StepView v = lbm::state_view(c, c->st.f_cur);
        unsigned char *d = host + (size_t)h * snap_bytes;
        const size_t b0 = sizeof(float) * n, bq = c->esz * (lbm::kQf - 1) * n, bg = c->esz * lbm::kQg * n;
        cudaError_t e = cudaMemcpyAsync(d, v.f0_in, b0, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d + b0, v.fq_in, bq, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d + b0 + bq, c->st.g, bg, cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess) return cuda_fail(e, "adjoint: host checkpoint");
        hsnaps[h].step = step;
        hsnaps[h].f_streamed = c->st.f_streamed;
        hsnaps[h].g_odd_next = c->st.g_odd_next;
        return LBM_OK;
    }

    // host slot h into device slot s (one copy: the layouts agree)
    int from_host(int h, int s)
    {
        cudaError_t e = cudaMemcpyAsync(slot_ptr(s), host + (size_t)h * snap_bytes, snap_bytes,
                                        cudaMemcpyHostToDevice, c->stream);
        if (e != cudaSuccess) return cuda_fail(e, "adjoint: host checkpoint restore");
        snaps[s] = hsnaps[h];
        return slot_ev.empty() ? LBM_OK : record(slot_ev[s], c->stream);
    }

    int restore(int s)
    {
        lbm::StepView v = lbm::state_view(c, 0);
        const unsigned char *d = slot_ptr(s);
        const size_t b0 = sizeof(float) * n, bq = c->esz * (lbm::kQf - 1) * n, bg = c->esz * lbm::kQg * n;
        cudaError_t e = cudaMemcpyAsync(c->st.f0, d, b0, cudaMemcpyDeviceToDevice, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(const_cast<void *>(v.fq_in), d + b0, bq, cudaMemcpyDeviceToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(c->st.g, d + b0 + bq, bg, cudaMemcpyDeviceToDevice, c->stream);
        if (e != cudaSuccess) return cuda_fail(e, "adjoint: restore");
        c->st.f_cur = 0;
        c->st.f_streamed = snaps[s].f_streamed;
        c->st.g_odd_next = snaps[s].g_odd_next;
        c->st.steps = snaps[s].step;
        return LBM_OK;
    }

    int forward(long long nsteps)
    {
        if (nsteps <= 0) return LBM_OK;
        fwd_steps += nsteps;
        return lbm_step(c, (int)nsteps, o.grav);
    }

    // One step of the state src (at step `step`) with its output in the
    // context (f half 0) or in slot `to`: checkpoints are read and written in
    // place, never copied through the context.
    int step_out_of_place(const lbm::NativeState &src, long long step, int to)
    {
        lbm::StepView v = lbm::state_view(c, 1);   // f out: half 0
        v.f0_in = src.f0;
        v.fq_in = src.fq;
        v.g_in = src.g;
        if (to >= 0) {
            unsigned char *d = slot_ptr(to);
            const size_t b0 = sizeof(float) * n, bq = c->esz * (lbm::kQf - 1) * n;
            v.f0_out = reinterpret_cast<float *>(d);
            v.fq_out = d + b0;
            v.g = d + b0 + bq;
        }
        cudaError_t e = lbm::launch_step(c->box, k, c->q, v, src.f_streamed, src.g_odd, false, c->stream);
        if (e != cudaSuccess) return cuda_fail(e, "adjoint: step kernel launch");
        fwd_steps++;
        if (to >= 0) {
            snaps[to].step = step + 1;
            snaps[to].f_streamed = false;
            snaps[to].g_odd_next = !src.g_odd;
            if (!slot_ev.empty()) return record(slot_ev[to], c->stream);
        } else {
            c->st.f_cur = 0;
            c->st.f_streamed = false;
            c->st.g_odd_next = !src.g_odd;
            c->st.steps = step + 1;
        }
        return LBM_OK;
    }

    // the context holds s^j, from s^s in slot si (j > s)
    int advance(int si, long long s, long long j)
    {
        int rc = step_out_of_place(slot_state(si), s, -1);
        if (!rc) rc = forward(j - s - 1);
        return rc ? rc : record(ctx_ev, c->stream);
    }

    // slot sj holds s^m, from s^s in slot si (m > s)
    int advance_to_slot(int si, long long s, long long m, int sj)
    {
        if (m - s == 1) return step_out_of_place(slot_state(si), s, sj);
        int rc = advance(si, s, m - 1);
        return rc ? rc : step_out_of_place(ctx_state(), m - 1, sj);
    }

    // phi of state st into buffer `out`, on stream `sm`
    int prepare(const lbm::NativeState &st, float *out, cudaStream_t sm)
    {
        cudaError_t e = lbm::launch_adjoint_phi(c->box, c->d.eta, c->q, st, out, sm);
        return e == cudaSuccess ? LBM_OK : cuda_fail(e, "adjoint: phi");
    }

    bool has_source(long long step) const { return step >= first_source; }

    // lambda^T from the final state (the context holds s^T), on the main
    // stream; the side stream starts after it
    int terminal()
    {
        const lbm::NativeState st = ctx_state();
        float *ph = phi_buf(o.nsteps);
        double *abT = ab_buf(o.nsteps);
        int rc = prepare(st, ph, c->stream);
        if (rc) return rc;
        cudaError_t e = cudaSuccess;
        if (has_source(o.nsteps)) {
            e = lbm::launch_objective(c->box, o.objective, c->d.phiStar, scale, c->q, st, ph, partials, abT, acc,
                                      c->stream);
            if (e == cudaSuccess)
                e = lbm::launch_source_init(c->box, o.objective, scale, abT, c->d.phiStar, c->q, st, ph, lam[cur],
                                            lam[cur] + lbm::kQf * n, lst[cur], c->stream);
        } else {
            e = cudaMemsetAsync(lam[cur], 0, sizeof(float) * (lbm::kQf + lbm::kQg) * n, c->stream);
            if (e == cudaSuccess) e = cudaMemsetAsync(lst[cur], 0, sizeof(float) * n, c->stream);
        }
        if (e != cudaSuccess) return cuda_fail(e, "adjoint: terminal source");
        if (side) {
            if ((rc = record(buf_free[o.nsteps & 1], c->stream))) return rc;
            e = cudaStreamWaitEvent(side, buf_free[o.nsteps & 1], 0);
            if (e != cudaSuccess) return cuda_fail(e, "adjoint: stream order");
        }
        lambda_ready = true;
        return LBM_OK;
    }

    // lambda^step from lambda^{step+1}; st is s^step, written when `ready` fires
    int adjoint_step(long long step, const lbm::NativeState &st, cudaEvent_t ready)
    {
        const bool src = has_source(step);
        float *ph = phi_buf(step);
        double *abs_ = ab_buf(step);
        const int b = (int)(step & 1);
        cudaError_t e = cudaStreamWaitEvent(side, ready, 0);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(side, buf_free[b], 0);
        if (e != cudaSuccess) return cuda_fail(e, "adjoint: stream order");
        int rc = prepare(st, ph, side);
        if (rc) return rc;
        if (src)
            e = lbm::launch_objective(c->box, o.objective, c->d.phiStar, scale, c->q, st, ph, partials, abs_, acc,
                                      side);
        if (e == cudaSuccess) e = cudaEventRecord(side_done, side);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, side_done, 0);
        if (e != cudaSuccess) return cuda_fail(e, "adjoint: side stream");
        lbm::AdjointBuffers a;
        a.phi = ph;
        a.lf_in = lam[cur];
        a.lg_in = lam[cur] + lbm::kQf * n;
        a.lst_in = lst[cur];
        a.lf_out = lam[1 - cur];
        a.lg_out = lam[1 - cur] + lbm::kQf * n;
        a.lst_out = lst[1 - cur];
        a.lsrc = lsrc;
        a.dgrav = dgrav;
        a.ab = abs_;
        e = lbm::launch_adjoint_step(c->box, k, c->d.phiStar, c->q, st, a, src, o.objective, scale, c->stream);
        if (e != cudaSuccess) return cuda_fail(e, "adjoint step");
        cur = 1 - cur;
        adj_steps++;
        return record(buf_free[b], c->stream);
    }

    // adjoint of step s (the segment [s, s + 1)); slot si holds s^s
    int leaf(long long s, int si)
    {
        int rc;
        if (!lambda_ready) {   // s + 1 == T: build lambda^T first
            if ((rc = advance(si, s, s + 1)) || (rc = terminal())) return rc;
        }
        return adjoint_step(s, slot_state(si), slot_ev[si]);
    }

    int take_slot()
    {
        if (free_slots.empty()) return -1;
        const int s = free_slots.back();
        free_slots.pop_back();
        return s;
    }

    // reverse [s, e) with s^s in slot si and `cfree` slots available
    int revolve(long long s, long long e, int si, int cfree)
    {
        const long long len = e - s;
        int rc;
        if (len <= 0) return LBM_OK;
        if (len == 1) return leaf(s, si);
        if (cfree == 0) {
            for (long long j = e - 1; j >= s; j--) {
                if (!lambda_ready) {
                    if ((rc = advance(si, s, o.nsteps)) || (rc = terminal())) return rc;
                }
                if (j == s) {
                    if ((rc = adjoint_step(j, slot_state(si), slot_ev[si]))) return rc;
                } else if ((rc = advance(si, s, j)) || (rc = adjoint_step(j, ctx_state(), ctx_ev))) {
                    return rc;
                }
            }
            return LBM_OK;
        }
        const long long m = s + split_point(len, cfree);
        const int sj = take_slot();
        if (sj < 0) return fail(LBM_ESTATE, "adjoint: checkpoint pool exhausted");
        if ((rc = advance_to_slot(si, s, m, sj))) return rc;
        if ((rc = revolve(m, e, sj, cfree - 1))) return rc;
        free_slots.push_back(sj);
        return revolve(s, m, si, cfree);
    }

    // Two tiers: the trajectory in K segments of L steps; the first forward
    // sweep leaves the start of every segment but the first and the last in
    // host memory (the last one's start is still in the context when the sweep
    // ends), then the segments are reversed last to first, each from its start
    // in a device base slot with the other device slots (segment 0 from slot 0,
    // which holds s^0, with all of them).  hslots host slots give K = hslots + 2
    // segments at most.  The host copies run on a copy stream beside the
    // compute: each sweep checkpoint goes out through one of two device slots
    // (a device copy on the main stream, then the host copy), and while a
    // segment is reversed the next segment's start comes back into the other
    // base slot.  With fewer than four device slots the copies are made on
    // the main stream, one base slot.
    int two_level(long long hslots, long long nslots)
    {
        const long long T = o.nsteps;
        const long long L = (T + hslots + 1) / (hslots + 2);   // ceil(T / (hslots + 2))
        const long long K = (T + L - 1) / L;
        hsnaps.assign((size_t)std::max<long long>(K - 2, 0), Snapshot());
        if (nslots < 4) return two_level_serial(T, L, K, nslots);
        int b[2] = {take_slot(), take_slot()};   // the sweep's outbound slots, then the segment bases
        if (b[0] < 0 || b[1] < 0) return fail(LBM_ESTATE, "adjoint: checkpoint pool exhausted");
        cudaStream_t cp = nullptr;
        cudaEvent_t saved = nullptr, done[2] = {nullptr, nullptr}, freed[2] = {nullptr, nullptr},
                    in[2] = {nullptr, nullptr};
        cudaError_t e = cudaStreamCreateWithFlags(&cp, cudaStreamNonBlocking);
        for (cudaEvent_t *x : {&saved, &done[0], &done[1], &freed[0], &freed[1], &in[0], &in[1]})
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(x, cudaEventDisableTiming);
        for (int i = 0; i < 2 && e == cudaSuccess; i++) {
            e = cudaEventRecord(done[i], cp);
            if (e == cudaSuccess) e = cudaEventRecord(freed[i], c->stream);
        }
        int rc = e == cudaSuccess ? LBM_OK : cuda_fail(e, "adjoint: host copy stream");
        auto wait = [&](cudaStream_t st, cudaEvent_t ev) {
            const cudaError_t w = cudaStreamWaitEvent(st, ev, 0);
            return w == cudaSuccess ? LBM_OK : cuda_fail(w, "adjoint: host copy order");
        };
        auto rec = [&](cudaEvent_t ev, cudaStream_t st) {
            const cudaError_t w = cudaEventRecord(ev, st);
            return w == cudaSuccess ? LBM_OK : cuda_fail(w, "adjoint: host copy order");
        };
        // sweep: s^{kL} of k = 1 .. K - 2 to host slot k - 1 through b[k & 1]
        for (long long k = 1; k < K && !rc; k++) {
            rc = forward(L);
            if (rc || k == K - 1) continue;
            const int i = (int)(k & 1);
            if (!(rc = wait(c->stream, done[i])) && !(rc = save(b[i], k * L)) && !(rc = rec(saved, c->stream)) &&
                !(rc = wait(cp, saved))) {
                e = cudaMemcpyAsync(host + (size_t)(k - 1) * snap_bytes, slot_ptr(b[i]), snap_bytes,
                                    cudaMemcpyDeviceToHost, cp);
                rc = e == cudaSuccess ? rec(done[i], cp) : cuda_fail(e, "adjoint: host checkpoint");
                hsnaps[(size_t)(k - 1)] = snaps[b[i]];
            }
        }
        // reverse: segment k from base b[cur]; segment k - 1's start comes into b[1 - cur] meanwhile
        int cur = 0;
        if (!rc && !(rc = wait(c->stream, done[0]))) rc = save(b[cur], (K - 1) * L);
        for (long long k = K - 1; k >= 1 && !rc; k--) {
            const bool next = k - 1 >= 1;
            const int nx = 1 - cur;
            if (next && !(rc = wait(cp, freed[nx])) && !(rc = wait(cp, done[nx]))) {
                e = cudaMemcpyAsync(slot_ptr(b[nx]), host + (size_t)(k - 2) * snap_bytes, snap_bytes,
                                    cudaMemcpyHostToDevice, cp);
                rc = e == cudaSuccess ? rec(in[nx], cp) : cuda_fail(e, "adjoint: host checkpoint restore");
                if (!rc) rc = rec(slot_ev[b[nx]], cp);
                snaps[b[nx]] = hsnaps[(size_t)(k - 2)];
            }
            if (!rc) rc = revolve(k * L, std::min(T, (k + 1) * L), b[cur], (int)(nslots - 3));
            if (!rc) rc = rec(freed[cur], c->stream);
            if (!rc && next) {
                rc = wait(c->stream, in[nx]);
                cur = nx;
            }
        }
        if (cp) cudaStreamSynchronize(cp);
        for (cudaEvent_t x : {saved, done[0], done[1], freed[0], freed[1], in[0], in[1]})
            if (x) cudaEventDestroy(x);
        if (cp) cudaStreamDestroy(cp);
        free_slots.push_back(b[1]);
        free_slots.push_back(b[0]);
        if (!rc) rc = revolve(0, std::min(T, L), 0, (int)(nslots - 1));
        return rc;
    }

    // the same with the host copies on the main stream and one base slot
    int two_level_serial(long long T, long long L, long long K, long long nslots)
    {
        const int base = take_slot();
        if (base < 0) return fail(LBM_ESTATE, "adjoint: checkpoint pool exhausted");
        int rc = LBM_OK;
        for (long long k = 1; k < K && !rc; k++) {
            rc = forward(L);                               // the context: s^{(k - 1) L} -> s^{k L}
            if (!rc && k < K - 1) rc = to_host((int)(k - 1), k * L);
        }
        if (!rc) rc = save(base, (K - 1) * L);
        for (long long k = K - 1; k >= 1 && !rc; k--) {
            if (k < K - 1) rc = from_host((int)(k - 1), base);
            if (!rc) rc = revolve(k * L, std::min(T, (k + 1) * L), base, (int)(nslots - 2));
        }
        free_slots.push_back(base);
        if (!rc) rc = revolve(0, std::min(T, L), 0, (int)(nslots - 1));
        return rc;
    }

    void release()
    {
        cudaStreamSynchronize(c->stream);
        if (side) {
            cudaStreamSynchronize(side);
            cudaStreamDestroy(side);
        }
        for (cudaEvent_t x : slot_ev)
            if (x) cudaEventDestroy(x);
        for (cudaEvent_t x : {ctx_ev, side_done, buf_free[0], buf_free[1]})
            if (x) cudaEventDestroy(x);
    }

    // the work buffers, carved from the context's arena; the objective alone
    // needs only phi, mom_save and the sums
    void carve(Carver &w, bool gradient, size_t nblocks)
    {
        phi = w.take<float>(2 * n);
        mom_save = w.take<float>(5 * n);
        partials = w.take<double>(2 * nblocks);
        ab = w.take<double>(8);
        acc = w.take<double>(2);
        if (!gradient) return;
        lam[0] = w.take<float>((size_t)(lbm::kQf + lbm::kQg) * n);
        lam[1] = w.take<float>((size_t)(lbm::kQf + lbm::kQg) * n);
        lst[0] = w.take<float>(n);
        lst[1] = w.take<float>(n);
        lsrc = w.take<float4>(n);
        phi0 = w.take<float>(n);
        dgrav = w.take<double>(lbm::adjoint_dgrav_parts(c->box));
    }
};

// Grow a cached device buffer to `need` bytes (a larger one is kept).
int ensure(void *&p, size_t &have, size_t need, const char *what)
{
    if (have >= need) return LBM_OK;
    cudaFree(p);
    p = nullptr;
    have = 0;
    cudaError_t e = cudaMalloc(&p, need);
    if (e != cudaSuccess) {
        p = nullptr;
        return cuda_fail(e, what);
    }
    have = need;
    return LBM_OK;
}

// The arena and the pool for one call: work buffers carved from
// c->adj_work, `slot_need` bytes of checkpoints in c->adj_slots.
int workspace(lbm_ctx *c, Adjoint &A, bool gradient, const char *fn)
{
    const size_t nblocks = lbm::adjoint_blocks(c->box);
    Carver dry{nullptr};
    A.carve(dry, gradient, nblocks);
    int rc = ensure(c->adj_work, c->adj_work_bytes, dry.off, fn);
    if (rc) return rc;
    Carver w{static_cast<unsigned char *>(c->adj_work)};
    A.carve(w, gradient, nblocks);
    return LBM_OK;
}

}  // namespace

namespace {

int check_opts(lbm_ctx *c, const lbm_adjoint_opts *o, const void *out, const char *fn)
{
    const std::string f(fn);
    if (!c || !o || !out) return fail(LBM_EINVAL, f + ": NULL argument");
    if (o->nsteps < 1) return fail(LBM_EINVAL, f + ": nsteps must be >= 1");
    if (o->objective != LBM_OBJ_LIGHT_UZ_MEAN && o->objective != LBM_OBJ_LIGHT_Z_CENTROID)
        return fail(LBM_EINVAL, f + ": unknown objective");
    if (o->objective == LBM_OBJ_LIGHT_UZ_MEAN && (o->window < 1 || o->window > o->nsteps))
        return fail(LBM_EINVAL, f + ": window must be in [1, nsteps]");
    if (!std::isfinite(o->grav)) return fail(LBM_EINVAL, f + ": grav is not finite");
    if (c->box.zghost) return fail(LBM_EINVAL, f + ": not available on a z-slab context");
    if (c->st.steps != 0)
        return fail(LBM_ESTATE, f + ": the context must hold its initial state (no step taken)");
    return LBM_OK;
}

void setup(Adjoint &A, lbm_ctx *c, const lbm_adjoint_opts *o)
{
    A.c = c;
    A.o = *o;
    A.n = (size_t)c->box.n;
    A.snap_bytes = sizeof(float) * A.n + c->esz * (lbm::kQf - 1 + lbm::kQg) * A.n;
    A.k = lbm::step_const(c->d, c->p, o->grav);
    A.first_source = o->objective == LBM_OBJ_LIGHT_UZ_MEAN ? o->nsteps - o->window + 1 : o->nsteps;
    A.scale = o->objective == LBM_OBJ_LIGHT_UZ_MEAN ? 1.0 / o->window : 1.0;
}

}  // namespace

extern "C" int lbm_objective(lbm_ctx *c, const lbm_adjoint_opts *o, double *J)
{
    const lbm::Range nvtx_range("lbm_objective");
    int rc = check_opts(c, o, J, "lbm_objective");
    if (rc) return rc;
    LBM_ON_DEVICE(c->p.device);
    Adjoint A;
    setup(A, c, o);
    const size_t n = A.n;
    if ((rc = workspace(c, A, false, "lbm_objective: work buffers")) ||
        (rc = ensure(c->adj_slots, c->adj_slot_bytes, A.snap_bytes, "lbm_objective: snapshot")))
        return rc;
    A.slots = static_cast<unsigned char *>(c->adj_slots);
    A.snaps.assign(1, Snapshot());
    cudaError_t e = cudaMemsetAsync(A.acc, 0, sizeof(double) * 2, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(A.mom_save, c->st.mom, sizeof(float) * 5 * n, cudaMemcpyDeviceToDevice, c->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "lbm_objective: setup");
    if (!rc) rc = A.save(0, 0);
    if (!rc) rc = A.forward(A.first_source);
    for (long long k = A.first_source; !rc && k <= o->nsteps; k++) {
        const lbm::NativeState st = A.ctx_state();
        rc = A.prepare(st, A.phi, c->stream);
        if (!rc) {
            e = lbm::launch_objective(c->box, o->objective, c->d.phiStar, A.scale, c->q, st, A.phi, A.partials, A.ab,
                                      A.acc, c->stream);
            if (e != cudaSuccess) rc = cuda_fail(e, "lbm_objective: objective");
        }
        if (!rc && k < o->nsteps) rc = A.forward(1);
    }
    double acc[2] = {0.0, 0.0};
    if (!rc) {
        e = cudaMemcpyAsync(acc, A.acc, sizeof(acc), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) rc = A.restore(0);
        if (e == cudaSuccess && !rc)
            e = cudaMemcpyAsync(c->st.mom, A.mom_save, sizeof(float) * 5 * n, cudaMemcpyDeviceToDevice, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess && !rc) rc = cuda_fail(e, "lbm_objective: results");
    }
    A.release();
    if (rc) return rc;
    *J = acc[0];
    return LBM_OK;
}

extern "C" int lbm_step_adjoint(lbm_ctx *c, const lbm_adjoint_opts *o, lbm_adjoint_out *out)
{
    const lbm::Range nvtx_range("lbm_step_adjoint");
    int rc0 = check_opts(c, o, out, "lbm_step_adjoint");
    if (rc0) return rc0;
    LBM_ON_DEVICE(c->p.device);
    const auto t0 = std::chrono::steady_clock::now();
    cudaError_t e = cudaSuccess;
    Adjoint A;
    setup(A, c, o);
    const size_t n = A.n;
    const size_t nblocks = lbm::adjoint_blocks(c->box);
    int rc = workspace(c, A, true, "lbm_step_adjoint: work buffers");
    if (rc) return rc;
    // checkpoint pool (a cached pool counts as free for the default budget)
    double budget = o->checkpoint_bytes;
    if (!(budget > 0)) {
        // the free device memory (the cached pool counted as free) less a
        // reserve of 5% of the device or 4 GiB, whichever is larger: every
        // checkpoint slot saves forward recomputation
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        const double reserve = std::max(4.0 * 1073741824.0, 0.05 * (double)tot);
        budget = (double)fr + (double)c->adj_slot_bytes - reserve;
    }
    long long nslots = (long long)(budget / (double)A.snap_bytes);
    nslots = std::min<long long>(nslots, (long long)o->nsteps + 1);
    if (nslots < 1)
        return fail(LBM_ENOMEM, "lbm_step_adjoint: checkpoint budget below one snapshot (" +
                                    std::to_string(A.snap_bytes) + " bytes)");
    if ((rc = ensure(c->adj_slots, c->adj_slot_bytes, (size_t)nslots * A.snap_bytes,
                     "lbm_step_adjoint: checkpoint pool")))
        return rc;
    A.slots = static_cast<unsigned char *>(c->adj_slots);
    A.snaps.assign((size_t)nslots, Snapshot());
    for (long long s = nslots - 1; s >= 1; s--) A.free_slots.push_back((int)s);
    // the second tier: pinned host slots for segment starts (two device slots
    // at least: s^0 and a segment's start)
    long long hslots = 0;
    if (o->host_checkpoint_bytes > 0 && nslots >= 2 && o->nsteps >= 3) {
        hslots = (long long)(o->host_checkpoint_bytes / (double)A.snap_bytes);
        hslots = std::min<long long>(hslots, (long long)o->nsteps - 2);
    }
    if (hslots >= 1 && c->adj_host_bytes < (size_t)hslots * A.snap_bytes) {
        if (c->adj_host) cudaFreeHost(c->adj_host);
        c->adj_host = nullptr;
        c->adj_host_bytes = 0;
        e = cudaHostAlloc(&c->adj_host, (size_t)hslots * A.snap_bytes, cudaHostAllocDefault);
        if (e != cudaSuccess) {
            c->adj_host = nullptr;
            return cuda_fail(e, "lbm_step_adjoint: host checkpoint pool");
        }
        c->adj_host_bytes = (size_t)hslots * A.snap_bytes;
    }
    A.host = static_cast<unsigned char *>(c->adj_host);

    e = cudaMemsetAsync(A.acc, 0, sizeof(double) * 2, c->stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(A.dgrav, 0, sizeof(double) * lbm::adjoint_dgrav_parts(c->box), c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(A.phi0, c->st.mom, sizeof(float) * n, cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(A.mom_save, c->st.mom, sizeof(float) * 5 * n, cudaMemcpyDeviceToDevice, c->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "lbm_step_adjoint: setup");
    if (!rc) rc = A.create_streams((int)nslots);
    if (!rc) rc = A.save(0, 0);
    if (!rc) rc = hslots >= 1 ? A.two_level(hslots, nslots) : A.revolve(0, o->nsteps, 0, (int)(nslots - 1));
    // lambda^0 -> dJ/dphi0 through the initial equilibrium (output in the
    // lsrc buffer, phi as the scratch for the Laplacian's adjoint)
    float *lphi0 = reinterpret_cast<float *>(A.lsrc);
    if (!rc) {
        e = lbm::launch_dgrav_fold(c->box, A.dgrav, A.acc, c->stream);
        if (e == cudaSuccess)
            e = lbm::launch_init_adjoint(c->box, c->d, c->p.Gamma, A.phi0, A.lam[A.cur], A.lst[A.cur],
                                         A.lam[A.cur] + lbm::kQf * n, lphi0, A.phi, c->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "lbm_step_adjoint: initial-state adjoint");
    }
    double acc[2] = {0.0, 0.0};
    if (!rc) {
        e = cudaMemcpyAsync(acc, A.acc, sizeof(acc), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess && out->dJ_dphi0)
            e = cudaMemcpyAsync(out->dJ_dphi0, lphi0, sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream);
        // leave the context at its initial state with its initial fields
        if (e == cudaSuccess) rc = A.restore(0);
        if (e == cudaSuccess && !rc)
            e = cudaMemcpyAsync(c->st.mom, A.mom_save, sizeof(float) * 5 * n, cudaMemcpyDeviceToDevice, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess && !rc) rc = cuda_fail(e, "lbm_step_adjoint: results");
    }
    A.release();
    if (rc) return rc;
    out->J = acc[0];
    out->dJ_dgrav = acc[1];
    out->slots = (int)nslots;
    out->forward_steps = A.fwd_steps;
    out->adjoint_steps = A.adj_steps;
    out->checkpoint_bytes_used = (double)nslots * (double)A.snap_bytes;
    out->host_slots = (int)A.hsnaps.size();
    out->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return LBM_OK;
}

extern "C" int lbm_adjoint_release(lbm_ctx *c)
{
    if (!c) return fail(LBM_EINVAL, "lbm_adjoint_release: NULL context");
    LBM_ON_DEVICE(c->p.device);
    const cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "lbm_adjoint_release");
    cudaFree(c->adj_work);
    cudaFree(c->adj_slots);
    if (c->adj_host) cudaFreeHost(c->adj_host);
    c->adj_work = c->adj_slots = c->adj_host = nullptr;
    c->adj_work_bytes = c->adj_slot_bytes = c->adj_host_bytes = 0;
    return LBM_OK;
}

extern "C" long long lbm_adjoint_forward_steps(long long nsteps, int slots)
{
    if (nsteps < 1 || slots < 1) return -1;
    const long long nslots = std::min<long long>(slots, nsteps + 1);
    bool terminal = true;
    return schedule_steps(nsteps, 0, nsteps, (int)(nslots - 1), terminal);
}

extern "C" long long lbm_adjoint_forward_steps_tiers(long long nsteps, int slots, long long host_slots)
{
    if (nsteps < 1 || slots < 1 || host_slots < 0) return -1;
    const long long nslots = std::min<long long>(slots, nsteps + 1);
    const long long hslots = nsteps >= 3 && nslots >= 2 ? std::min(host_slots, nsteps - 2) : 0;
    if (hslots < 1) return lbm_adjoint_forward_steps(nsteps, slots);
    // the accounting of Adjoint::two_level: the sweep, then the segments
    // last to first from their base slots (two of them from four device slots
    // up, one below), then segment 0 from slot 0 with all the others
    const long long T = nsteps;
    const long long L = (T + hslots + 1) / (hslots + 2);
    const long long K = (T + L - 1) / L;
    const int cfree = (int)(nslots >= 4 ? nslots - 3 : nslots - 2);
    bool terminal = true;
    long long steps = (K - 1) * L;
    for (long long k = K - 1; k >= 1; k--) steps += schedule_steps(T, k * L, std::min(T, (k + 1) * L), cfree, terminal);
    return steps + schedule_steps(T, 0, std::min(T, L), (int)(nslots - 1), terminal);
}
