// hfx_session.cpp -- multi-job Fock session: every SCF cycle, one launch per
// quartet class over the quartets of all member jobs.
//
// The reference solves one molecule at a time (run.hpp:300-423); its GPU
// path launches one kernel per ERI tensor (cuda/src/eri.cu:20-89).  Here the
// request server's packed mode keeps a session per (method, options, size
// class): each request builds its own job (pair records, Schwarz table,
// launch plans) on its worker thread, joins the session, and from its next
// SCF cycle on its quartets are part of the session's launches.
//
// Layout.  The members' device tables stay where their jobs put them.  The
// session builds a combined pair table whose records address every member's
// arrays as anchor + offset (the offsets are taken in the device's single
// address space; anchor64_ / anchor32_ are small session allocations), with
// the member's matrices at its own offset of the session's packed density /
// accumulator / output buffers and its pair indices shifted to its block of
// the combined table.  The members' launch-group task lists are concatenated
// per class (small classes by bra/ket class and precision, the warp kernel by
// precision and shared-memory tier) and their pair indices shifted by a
// device pass.  The layout is rebuilt whenever a member joins or leaves.
//
// Cycle.  A member that needs a build waits until every live member has
// asked; the last one runs the session's builds -- one per distinct
// (precision plan, density screening) variant among the requests, each with
// only that variant's members switched on -- staging each member's densities
// in and copying its results out, then wakes the others.
#include "hfx_session.hpp"

#include <algorithm>
#include <cstdint>
#include <cstring>

namespace hfx {

static long long elem_offset(const void* p, const void* anchor, size_t elem)
{
    const long long d = (long long)((intptr_t)p - (intptr_t)anchor);
    if (d % (long long)elem != 0) throw Error(HFX_ERR_CUDA, "session: misaligned member table");
    return d / (long long)elem;
}

FockSession::FockSession(int device, int nspin, double screening_threshold)
    : device_(device), nspin_(nspin), thr_(screening_threshold)
{
    if (nspin != 1 && nspin != 2) throw Error(HFX_ERR_INVALID, "session: nspin must be 1 or 2");
    if (thr_ == 0.0) thr_ = 1e-8;
    cuda_check(cudaSetDevice(device_), "cudaSetDevice");
    cuda_check(cudaDeviceGetAttribute(&nsm_, cudaDevAttrMultiProcessorCount, device_), "SM count");
    cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
    for (int s = 0; s < 3; ++s) {
        cudaStream_t st;
        cuda_check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
        aux_.push_back(st);
        cudaEvent_t ev;
        cuda_check(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event");
        aux_ev_.push_back(ev);
    }
    cuda_check(cudaEventCreateWithFlags(&fork_ev_, cudaEventDisableTiming), "event");
    cuda_check(cudaEventCreate(&ev0_), "event");
    cuda_check(cudaEventCreate(&ev1_), "event");
    anchor64_.alloc(32);
    anchor32_.alloc(64);
    boys64_.upload(boys_table64_host(), stream_);
    boys32_.upload(boys_table32_host(), stream_);
    const ClassTables& ct = class_tables();
    pct_.upload(ct.tab, stream_);
    abs_.upload(ct.ab_start, stream_);
    kh_.upload(ct.k_herm, stream_);
    kl_.upload(ct.k_lin, stream_);
    cuda_check(cudaStreamSynchronize(stream_), "session setup");
}

FockSession::~FockSession()
{
    cudaSetDevice(device_);
    if (stream_) cudaStreamSynchronize(stream_);
    for (auto e : aux_ev_) cudaEventDestroy(e);
    for (auto st : aux_) cudaStreamDestroy(st);
    if (fork_ev_) cudaEventDestroy(fork_ev_);
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
    if (stream_) cudaStreamDestroy(stream_);
}

int FockSession::members() const
{
    std::lock_guard<std::mutex> lk(mu_);
    int n = 0;
    for (const Member& m : slots_) n += m.live ? 1 : 0;
    return n;
}

int FockSession::join(Job& job)
{
    if (job.device() != device_) throw Error(HFX_ERR_INVALID, "session: job on another device");
    if (job.opt_.screening_threshold != thr_) throw Error(HFX_ERR_INVALID, "session: screening threshold differs");
    if (job.fragments().count() != 1) throw Error(HFX_ERR_INVALID, "session: packed jobs cannot join");
    std::lock_guard<std::mutex> lk(mu_);
    if (failed_) throw Error(fail_code_, fail_msg_);
    int slot = -1;
    for (size_t s = 0; s < slots_.size(); ++s)
        if (!slots_[s].live) {
            slot = (int)s;
            break;
        }
    if (slot < 0) {
        slot = (int)slots_.size();
        slots_.emplace_back();
    }
    slots_[slot] = Member{};
    slots_[slot].job = &job;
    slots_[slot].live = true;
    dirty_ = true;
    int n = 0;
    for (const Member& m : slots_) n += m.live ? 1 : 0;
    max_members_ = std::max(max_members_, n);
    return slot;
}

void FockSession::leave(int slot)
{
    std::lock_guard<std::mutex> lk(mu_);
    if (slot < 0 || slot >= (int)slots_.size() || !slots_[slot].live) return;
    slots_[slot].live = false;
    slots_[slot].job = nullptr;
    dirty_ = true;
    int n = 0;
    for (const Member& m : slots_) n += m.live ? 1 : 0;
    // the members already waiting no longer wait for this one
    if (!pending_.empty() && (int)pending_.size() == n) run_locked();
}

void FockSession::build(int slot, cudaStream_t st, const double* dPa, const double* dPb, double* o0, double* o1,
                        double* o2, bool mixed, double dthr, double* ms)
{
    cuda_check(cudaStreamSynchronize(st), "session: member densities");
    std::unique_lock<std::mutex> lk(mu_);
    if (failed_) throw Error(fail_code_, fail_msg_);
    if (slot < 0 || slot >= (int)slots_.size() || !slots_[slot].live) throw Error(HFX_ERR_INVALID, "session: not a member");
    pending_.push_back(Req{slot, dPa, dPb, o0, o1, o2, mixed, dthr});
    const unsigned long long gen = generation_;
    int n = 0;
    for (const Member& m : slots_) n += m.live ? 1 : 0;
    if ((int)pending_.size() == n)
        run_locked();
    else
        cv_.wait(lk, [&] { return generation_ != gen; });
    if (failed_) throw Error(fail_code_, fail_msg_);
    if (ms) *ms = cycle_ms_;
}

void FockSession::relayout()
{
    live_.clear();
    for (size_t s = 0; s < slots_.size(); ++s)
        if (slots_[s].live) live_.push_back((int)s);
    nmat_ = 0;
    npairs_ = 0;
    std::vector<DPair> h64, h32;
    std::vector<int> fk;
    std::vector<long long> fm;
    lane_min_npp_ = -1;
    for (size_t f = 0; f < live_.size(); ++f) {
        Member& m = slots_[live_[f]];
        Job& j = *m.job;
        m.frag = (int)f;
        m.moff = nmat_;
        m.pair_off = npairs_;
        const int K = j.K();
        nmat_ += (long long)K * K;
        const long long d64 = elem_offset(j.d_rec64_.p, anchor64_.p, sizeof(double));
        const long long d32 = elem_offset(j.d_rec32_.p, anchor32_.p, sizeof(float));
        const long long dq = elem_offset(j.d_qbf_.p, anchor64_.p, sizeof(double));
        const long long dq32 = elem_offset(j.d_qbf32_.p, anchor32_.p, sizeof(float));
        for (const DPair& src : j.dpairs_host_) {
            DPair x = src;
            x.moff = m.moff;
            x.qoff = dq + src.qoff;
            x.pbase = m.pair_off + src.pbase;
            x.id = m.pair_off + src.id;
            x.frag = (int)f;
            x.kdim = K;
            DPair a = x, b = x;
            a.rec_off = d64 + src.rec_off;
            b.rec_off = d32 + src.rec_off;
            b.qoff = dq32 + src.qoff;   // the FP32 kernels screen with the float table
            h64.push_back(a);
            h32.push_back(b);
        }
        npairs_ += (int)j.dpairs_host_.size();
        fk.push_back(K);
        fm.push_back(m.moff);
        const int lm = j.shape_.lane_min_npp;
        lane_min_npp_ = lane_min_npp_ < 0 ? lm : (lane_min_npp_ == lm ? lm : 0);
    }
    if (lane_min_npp_ < 0) lane_min_npp_ = kDefaultLaneMinNpp;
    if (live_.empty()) {
        plan64_.groups.clear();
        plan_mixed_.groups.clear();
        dirty_ = false;
        return;
    }
    pairs64_.upload(h64, stream_);
    pairs32_.upload(h32, stream_);
    fk_.upload(fk, stream_);
    fmoff_.upload(fm, stream_);
    active_.alloc(live_.size());
    const size_t n = (size_t)nmat_;
    for (int s = 0; s < nspin_; ++s) in_[s].alloc(n);
    if (nspin_ == 2) dj_.alloc(n);
    for (int s = 0; s < nspin_ + 1; ++s) acc_[s].alloc(n);
    for (int s = 0; s < 2 * nspin_ - 1; ++s) out_[s].alloc(n);
    dsh_.alloc((size_t)std::max(1, npairs_));
    d32_.alloc(3 * n);
    combine(false, plan64_);
    combine(true, plan_mixed_);
    counters_.alloc(std::max<size_t>(1, std::max(plan64_.groups.size(), plan_mixed_.groups.size())));
    cuda_check(cudaStreamSynchronize(stream_), "session layout");
    dirty_ = false;
}

// The members' launch groups of one plan, merged by class: small classes by
// (bra class, ket class, precision), the warp kernel by (precision,
// shared-memory tier); task lists concatenated, pair indices shifted.
void FockSession::combine(bool mixed_plan, Combined& c)
{
    struct Part {
        int member;
        const GroupSet* gs;
        const LaunchGroup* g;
    };
    std::map<std::tuple<int, int, int, int>, std::vector<Part>> parts;
    for (size_t f = 0; f < live_.size(); ++f) {
        const Job& j = *slots_[live_[f]].job;
        const GroupSet& gs = j.plan(mixed_plan);
        for (const LaunchGroup& g : gs.groups) {
            if (g.n == 0) continue;
            int tier = 0;
            if (g.kind == 1)
                while ((512 << tier) < g.slice) ++tier;
            auto key = g.kind == 0 ? std::make_tuple(0, g.pcb, g.pck, g.fp32 ? 1 : 0)
                                   : std::make_tuple(1, g.fp32 ? 1 : 0, tier, 0);
            parts[key].push_back(Part{live_[f], &gs, &g});
        }
    }
    size_t total = 0;
    for (auto& kv : parts)
        for (const Part& p : kv.second) total += p.g->n;
    c.groups.clear();
    c.tasks.alloc(std::max<size_t>(1, total));
    size_t off = 0;
    const size_t elem[2] = {sizeof(double), sizeof(float)};
    for (auto& kv : parts) {
        LaunchGroup cg{};
        const LaunchGroup& g0 = *kv.second.front().g;
        cg.kind = g0.kind;
        cg.pcb = g0.pcb;
        cg.pck = g0.pck;
        cg.fp32 = g0.fp32;
        cg.off = off;
        for (const Part& p : kv.second) {
            const LaunchGroup& g = *p.g;
            cuda_check(cudaMemcpyAsync(c.tasks.p + off, p.gs->tasks.p + g.off, g.n * sizeof(Task),
                                       cudaMemcpyDeviceToDevice, stream_),
                       "session tasks");
            Task* t = c.tasks.p + off;
            long long nt = (long long)g.n;
            int delta = slots_[p.member].pair_off;
            if (delta != 0) {
                KernelSpec ks = rebase_tasks_spec(nt);
                void* prm[] = {&t, &nt, &delta};
                cuda_check(cudaLaunchKernel(ks.func, ks.grid, ks.block, prm, 0, stream_), "session rebase");
            }
            off += g.n;
            cg.n += g.n;
            cg.flops += g.flops;
            cg.prims += g.prims;
            cg.slice = std::max(cg.slice, g.slice);
        }
        if (cg.kind == 1) {
            const int f = cg.fp32 ? 1 : 0;
            cg.slice = (cg.slice + 1) & ~1;
            cg.lane_min_npp = lane_min_npp_;
            cg.warps_per_cta = (int)std::max<size_t>(
                1, std::min<size_t>(8, (200 * 1024 - kWarpSmemHeader) / ((size_t)cg.slice * elem[f])));
            const size_t sm = kWarpSmemHeader + elem[f] * (size_t)cg.slice * cg.warps_per_cta;
            const int ctas_per_sm = (int)std::max<size_t>(1, (228 * 1024) / (sm + 1024));
            const long long need = ((long long)cg.n + cg.warps_per_cta - 1) / cg.warps_per_cta;
            cg.grid = (int)std::min<long long>(need, (long long)nsm_ * ctas_per_sm);
        }
        c.groups.push_back(cg);
    }
}

// One build of the live members switched on in active_ (J/K into acc_,
// symmetrised into out_), on the session's streams.
void FockSession::launch(int nk, bool mixed_plan, double dthr)
{
    const Combined& c = mixed_plan ? plan_mixed_ : plan64_;
    const size_t n = (size_t)nmat_;
    StreamSink sk(stream_, aux_, fork_ev_, aux_ev_);
    for (int s = 0; s < nk + 1; ++s) sk.zero(0, acc_[s].p, n * sizeof(double));
    const double* Dj = in_[0].p;
    const double* Dk = in_[0].p;
    const double* Dk2 = nullptr;
    if (nk == 2) {
        const double* a = in_[0].p;
        const double* b = in_[1].p;
        double* d = dj_.p;
        long long nn = (long long)n;
        void* prm[] = {&a, &b, &d, &nn};
        sk.kernel(0, add_spec(nn), prm);
        Dj = dj_.p;
        Dk2 = in_[1].p;
    }
    double* J = acc_[0].p;
    double* Kx = acc_[1].p;
    double* Kx2 = nk == 2 ? acc_[2].p : nullptr;
    const double* Dsh = nullptr;
    if (dthr > 0.0 && npairs_ > 0) {
        const DPair* pr = pairs64_.p;
        int np = npairs_;
        double* out = dsh_.p;
        void* prm[] = {&pr, &np, &Dk, &Dk2, &out};
        sk.kernel(0, density_blocks_spec(np), prm);
        Dsh = dsh_.p;
    }
    const float *Dj32 = nullptr, *Dk32 = nullptr, *Dk232 = nullptr;
    bool any32 = false;
    for (const auto& g : c.groups) any32 = any32 || g.fp32;
    if (any32) {
        long long nn = (long long)n;
        const double* src[3] = {Dj, Dk, Dk2};
        const float* dst[3] = {nullptr, nullptr, nullptr};
        for (int s = 0; s < 3; ++s) {
            if (!src[s]) continue;
            int same = -1;
            for (int q = 0; q < s; ++q)
                if (src[q] == src[s]) same = q;
            if (same >= 0) {
                dst[s] = dst[same];
                continue;
            }
            const double* in = src[s];
            float* out = d32_.p + (size_t)s * n;
            void* prm[] = {&in, &out, &nn};
            sk.kernel(0, to_float_spec(nn), prm);
            dst[s] = out;
        }
        Dj32 = dst[0];
        Dk32 = dst[1];
        Dk232 = dst[2];
    }
    const unsigned char* active = active_.p;
    int* ctr = counters_.p;
    sk.zero(0, ctr, sizeof(int) * std::max<size_t>(1, c.groups.size()));
    sk.fork();
    const Task* tasks = c.tasks.p;
    const int naux = (int)aux_.size();
    int next_aux = 0;
    for (size_t gi = 0; gi < c.groups.size(); ++gi) {
        const LaunchGroup& g = c.groups[gi];
        KernelSpec ks;
        if (g.kind == 0) {
            const int lane = 1 + next_aux;
            next_aux = (next_aux + 1) % naux;
            if (g.fp32) {
                SmallArgs<float> a{pairs32_.p, anchor32_.p, tasks + g.off, (int)g.n, boys32_.p, thr_, nullptr,
                                   0, Dj, Dk, Dk2, J, Kx, Kx2, Dsh, dthr, active, Dj32, Dk32, Dk232, anchor32_.p};
                cuda_check(small_spec_f32(g.pcb, g.pck, nk, (int)g.n, &ks), "session small-class kernel");
                void* prm[] = {&a};
                sk.kernel(lane, ks, prm);
            } else {
                SmallArgs<double> a{pairs64_.p, anchor64_.p, tasks + g.off, (int)g.n, boys64_.p, thr_, anchor64_.p,
                                    0, Dj, Dk, Dk2, J, Kx, Kx2, Dsh, dthr, active, nullptr, nullptr, nullptr};
                cuda_check(small_spec_f64(g.pcb, g.pck, nk, (int)g.n, &ks), "session small-class kernel");
                void* prm[] = {&a};
                sk.kernel(lane, ks, prm);
            }
        } else {
            cuda_check(warp_spec(g.fp32, nk, g.grid, g.warps_per_cta, g.slice, &ks), "session warp kernel");
            if (g.fp32) {
                WarpArgs<float> a{pairs32_.p, anchor32_.p, pct_.p, abs_.p, kh_.p, kl_.p, tasks + g.off, (int)g.n,
                                  ctr + gi, boys32_.p, thr_, nullptr, 0, Dj, Dk, Dk2, J, Kx, Kx2, g.slice,
                                  g.lane_min_npp, Dsh, dthr, nullptr, nullptr, active, Dj32, Dk32, Dk232, anchor32_.p};
                void* prm[] = {&a};
                sk.kernel(0, ks, prm);
            } else {
                WarpArgs<double> a{pairs64_.p, anchor64_.p, pct_.p, abs_.p, kh_.p, kl_.p, tasks + g.off, (int)g.n,
                                   ctr + gi, boys64_.p, thr_, anchor64_.p, 0, Dj, Dk, Dk2, J, Kx, Kx2, g.slice,
                                   g.lane_min_npp, Dsh, dthr, nullptr, nullptr, active, nullptr, nullptr, nullptr};
                void* prm[] = {&a};
                sk.kernel(0, ks, prm);
            }
        }
    }
    sk.join();
    int kmax = 0;
    for (int s : live_) kmax = std::max(kmax, slots_[s].job->K());
    const int* fk = fk_.p;
    const long long* fm = fmoff_.p;
    const int nf = (int)live_.size();
    if (nk == 1) {
        const double* jp = acc_[0].p;
        const double* kp = acc_[1].p;
        double* G = out_[0].p;
        void* prm[] = {&jp, &kp, &G, &fk, &fm, &active};
        sk.kernel(0, finish_rhf_spec(kmax, nf), prm);
    } else {
        const double* jp = acc_[0].p;
        const double* kp = acc_[1].p;
        const double* k2 = acc_[2].p;
        double* o0 = out_[0].p;
        double* o1 = out_[1].p;
        double* o2 = out_[2].p;
        void* prm[] = {&jp, &kp, &k2, &o0, &o1, &o2, &fk, &fm, &active};
        sk.kernel(0, finish_uhf_spec(kmax, nf), prm);
    }
}

void FockSession::run_locked()
{
    double ms = 0.0;
    try {
        cuda_check(cudaSetDevice(device_), "cudaSetDevice");
        if (dirty_) relayout();
        std::map<std::pair<bool, double>, std::vector<const Req*>> variants;
        for (const Req& r : pending_) variants[{r.mixed, r.dthr}].push_back(&r);
        std::vector<unsigned char> flags(live_.size());
        for (const auto& kv : variants) {
            std::fill(flags.begin(), flags.end(), 0);
            for (const Req* r : kv.second) {
                const Member& m = slots_[r->slot];
                flags[m.frag] = 1;
                const size_t bytes = sizeof(double) * (size_t)m.job->K() * m.job->K();
                cuda_check(cudaMemcpyAsync(in_[0].p + m.moff, r->Pa, bytes, cudaMemcpyDeviceToDevice, stream_),
                           "session stage");
                if (nspin_ == 2)
                    cuda_check(cudaMemcpyAsync(in_[1].p + m.moff, r->Pb, bytes, cudaMemcpyDeviceToDevice, stream_),
                               "session stage");
            }
            cuda_check(cudaMemcpyAsync(active_.p, flags.data(), flags.size(), cudaMemcpyHostToDevice, stream_),
                       "session flags");
            cuda_check(cudaEventRecord(ev0_, stream_), "event");
            launch(nspin_, kv.first.first, kv.first.second);
            cuda_check(cudaEventRecord(ev1_, stream_), "event");
            for (const Req* r : kv.second) {
                const Member& m = slots_[r->slot];
                const size_t bytes = sizeof(double) * (size_t)m.job->K() * m.job->K();
                double* outs[3] = {r->o0, r->o1, r->o2};
                for (int s = 0; s < 2 * nspin_ - 1; ++s)
                    cuda_check(cudaMemcpyAsync(outs[s], out_[s].p + m.moff, bytes, cudaMemcpyDeviceToDevice, stream_),
                               "session results");
            }
            cuda_check(cudaStreamSynchronize(stream_), "session build");
            float t = 0.f;
            cudaEventElapsedTime(&t, ev0_, ev1_);
            ms += t;
            ++builds_;
        }
    } catch (const Error& e) {
        failed_ = true;
        fail_code_ = e.code;
        fail_msg_ = e.what();
    } catch (const std::exception& e) {
        failed_ = true;
        fail_code_ = HFX_ERR_CUDA;
        fail_msg_ = e.what();
    }
    cycle_ms_ = ms;
    build_ms_ += ms;
    pending_.clear();
    ++generation_;
    cv_.notify_all();
}

}  // namespace hfx
