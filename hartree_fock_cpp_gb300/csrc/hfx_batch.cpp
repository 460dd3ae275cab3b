// hfx_batch.cpp -- lockstep batched SCF over a packed job.
//
// The reference solves the geometries of a scan one after another
// (run_bl_scan, run.hpp:300-423; run_dissociation, run.hpp:498-577), each
// SCF with its own ERI pass.  Here all molecules of a batch share one packed
// job (hfx_engine.hpp: Job over several molecules, quartets never mixing
// molecules, matrices packed back to back), and their SCFs advance in
// lockstep: every cycle is ONE Fock build over every molecule still
// iterating -- one launch per quartet class over all molecules' quartets,
// replayed as a CUDA graph -- while each molecule's O(K^3) SCF steps
// (orthogonalisation, eigensolve, DIIS) run on its own stream and host thread
// through the same DeviceScf as a single job.
//
// Cycle protocol (PackedBuilder): a molecule thread stages its density into
// its block of the packed input, arrives, and sleeps; the last of the joined
// molecules to arrive (or to leave) runs the packed build for everyone --
// one build per distinct (precision plan, density screening) variant among
// the arrivals, each with only that variant's molecules switched on -- then
// wakes the others, who copy their blocks of the results.  Molecules
// join when their setup is done and leave when their SCF ends, so a batch
// larger than max_parallel streams through the packed job.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <tuple>

#include "hfx_batch.hpp"
#include "hfx_dscf.hpp"
#include "hfx_engine.hpp"

namespace hfx {

void set_last_error(const std::string& msg);

namespace {

constexpr double kBatchDeltaThr = 1e-12;   // density screening of incremental FP64 builds

class PackedBuilder {
public:
    PackedBuilder(Job& job, int nspin) : job_(job), nspin_(nspin)
    {
        const size_t n = (size_t)job.nmat();
        for (int s = 0; s < nspin; ++s) in_[s].alloc(n);
        for (int s = 0; s < 2 * nspin - 1; ++s) {
            out_[s].alloc(n);
            res_[s].alloc(n);
        }
        flags_.assign(job.fragments().count(), 0);
    }

    void join()
    {
        std::lock_guard<std::mutex> lk(mu_);
        ++participants_;
    }

    void leave()
    {
        std::unique_lock<std::mutex> lk(mu_);
        --participants_;
        if (!pending_.empty() && (int)pending_.size() == participants_) run_locked();
    }

    // One molecule's build of this cycle: stage, wait for the packed build, copy out.
    void build(int frag, cudaStream_t st, const double* dPa, const double* dPb, double* o0, double* o1, double* o2,
               bool mixed, double dthr, double* ms)
    {
        const Fragments& fr = job_.fragments();
        const long long off = fr.moff[frag];
        const size_t bytes = sizeof(double) * (size_t)fr.K(frag) * fr.K(frag);
        cuda_check(cudaMemcpyAsync(in_[0].p + off, dPa, bytes, cudaMemcpyDeviceToDevice, st), "stage density");
        if (nspin_ == 2)
            cuda_check(cudaMemcpyAsync(in_[1].p + off, dPb, bytes, cudaMemcpyDeviceToDevice, st), "stage density");
        cuda_check(cudaStreamSynchronize(st), "stage density");
        {
            std::unique_lock<std::mutex> lk(mu_);
            if (failed_) throw Error(fail_code_, fail_msg_);
            pending_.push_back({frag, mixed, dthr});
            const unsigned long long gen = generation_;
            if ((int)pending_.size() == participants_)
                run_locked();
            else
                cv_.wait(lk, [&] { return generation_ != gen; });
            if (failed_) throw Error(fail_code_, fail_msg_);
            *ms = cycle_ms_;
        }
        double* outs[3] = {o0, o1, o2};
        for (int s = 0; s < 2 * nspin_ - 1; ++s)
            cuda_check(cudaMemcpyAsync(outs[s], res_[s].p + off, bytes, cudaMemcpyDeviceToDevice, st), "fetch result");
        cuda_check(cudaStreamSynchronize(st), "fetch result");
    }

    int builds() const { return builds_; }
    double build_ms() const { return build_ms_; }

private:
    struct Req {
        int frag;
        bool mixed;
        double dthr;
    };

    // Runs the cycle's packed builds (mu_ held), then wakes the waiting molecules.
    void run_locked()
    {
        std::map<std::pair<bool, double>, std::vector<int>> variants;
        for (const Req& r : pending_) variants[{r.mixed, r.dthr}].push_back(r.frag);
        double ms = 0.0;
        try {
            for (const auto& kv : variants) {
                std::fill(flags_.begin(), flags_.end(), 0);
                for (int f : kv.second) flags_[f] = 1;
                job_.set_active(flags_.data());
                if (nspin_ == 1)
                    job_.fock_rhf_device_ex(in_[0].p, out_[0].p, kv.first.first, kv.first.second);
                else
                    job_.fock_uhf_device_ex(in_[0].p, in_[1].p, out_[0].p, out_[1].p, out_[2].p, kv.first.first,
                                            kv.first.second);
                ms += job_.stats.ms;
                ++builds_;
                // the variant's blocks to the result buffers before the next
                // variant's build reuses the packed outputs
                const Fragments& fr = job_.fragments();
                for (int f : kv.second) {
                    const size_t bytes = sizeof(double) * (size_t)fr.K(f) * fr.K(f);
                    for (int s = 0; s < 2 * nspin_ - 1; ++s)
                        cuda_check(cudaMemcpyAsync(res_[s].p + fr.moff[f], out_[s].p + fr.moff[f], bytes,
                                                   cudaMemcpyDeviceToDevice, job_.stream()),
                                   "gather results");
                }
                cuda_check(cudaStreamSynchronize(job_.stream()), "gather results");
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

    Job& job_;
    int nspin_;
    DevBuf<double> in_[2], out_[3], res_[3];
    std::vector<unsigned char> flags_;
    std::mutex mu_;
    std::condition_variable cv_;
    std::vector<Req> pending_;
    int participants_ = 0;
    unsigned long long generation_ = 0;
    bool failed_ = false;
    hfx_status fail_code_ = HFX_OK;
    std::string fail_msg_;
    double cycle_ms_ = 0.0, build_ms_ = 0.0;
    int builds_ = 0;
};

// One molecule's view of the packed job, as the device SCF sees a builder.
class BatchMember final : public FockSource {
public:
    BatchMember(PackedBuilder& b, int frag, int K, bool mixed) : b_(b), frag_(frag), K_(K), mixed_(mixed)
    {
        cuda_check(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking), "cudaStreamCreate");
    }
    ~BatchMember() override
    {
        if (st_) {
            cudaStreamSynchronize(st_);
            cudaStreamDestroy(st_);
        }
    }
    int K() const override { return K_; }
    cudaStream_t stream() const override { return st_; }
    bool mixed() const override { return mixed_; }
    void fock_rhf_device_ex(const double* dP, double* dG, bool mixed, double dthr) override
    {
        b_.build(frag_, st_, dP, nullptr, dG, nullptr, nullptr, mixed, dthr, &ms_);
    }
    void fock_uhf_device_ex(const double* dPa, const double* dPb, double* dJ, double* dKa, double* dKb, bool mixed,
                            double dthr) override
    {
        b_.build(frag_, st_, dPa, dPb, dJ, dKa, dKb, mixed, dthr, &ms_);
    }
    double last_build_ms() const override { return ms_; }

private:
    PackedBuilder& b_;
    int frag_, K_;
    bool mixed_;
    cudaStream_t st_ = nullptr;
    double ms_ = 0.0;
};

void fill(const ScfOutput& o, hfx_scf_result* r)
{
    std::memset(r, 0, sizeof(*r));
    r->E_tot = o.E_tot;
    r->E_ele = o.E_ele;
    r->E_nuc = o.E_nuc;
    r->iterations = o.iterations;
    r->converged = o.converged ? 1 : 0;
    r->K = o.K;
    r->n_electrons = o.n_electrons;
    r->seconds = o.seconds;
    r->fock_ms = o.fock_ms;
    r->fock_builds = o.fock_builds;
    r->mixed_builds = o.mixed_builds;
    r->fp64_builds = o.fp64_builds;
    r->delta_builds = o.delta_builds;
    r->projections = o.projections;
    r->projection_fallbacks = o.projection_fallbacks;
}

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

PackedRunStats run_packed(const std::vector<Basis>& bases, const hfx_options& jo, int nspin,
                          const std::vector<PackedMember>& members, int max_parallel, const PackedDone& done)
{
    const int n = (int)bases.size();
    if (n == 0) return PackedRunStats{};
    if ((int)members.size() != n) throw Error(HFX_ERR_INVALID, "packed run: one member spec per molecule");
    const double t0 = now_s();
    Job job(bases, jo);
    PackedBuilder builder(job, nspin);
    const double t_setup = now_s() - t0;
    // chains of consecutive molecules linked by warm_from (a molecule with
    // warm_from == -1 starts a new chain)
    std::vector<std::vector<int>> chains;
    for (int i = 0; i < n; ++i) {
        if (members[i].warm_from >= 0 && members[i].warm_from != i - 1)
            throw Error(HFX_ERR_INVALID, "packed run: a molecule can only start from the preceding one's density");
        if (members[i].warm_from < 0 || chains.empty()) chains.emplace_back();
        chains.back().push_back(i);
    }
    const int nchains = (int)chains.size();
    const int workers = std::max(1, std::min({nchains, max_parallel > 0 ? max_parallel : nchains, 256}));
    std::atomic<int> next{0};
    int dev = 0;
    cudaGetDevice(&dev);
    auto worker = [&] {
        cudaSetDevice(dev);
        for (int c = next++; c < nchains; c = next++) {
            std::vector<double> prevA, prevB;   // final densities of the chain's previous molecule
            for (int i : chains[c]) {
                bool joined = false;
                // warm start only from a density of this molecule's size
                const bool warm = members[i].warm_from >= 0 && !prevA.empty() &&
                                  prevA.size() == (size_t)bases[i].K * bases[i].K &&
                                  (nspin == 1 || prevB.size() == prevA.size());
                try {
                    const PackedMember& m = members[i];
                    ScfSetup setup = scf_setup(bases[i], true);
                    BatchMember member(builder, i, bases[i].K, job.mixed());
                    DeviceScf d(member, setup, nspin);
                    builder.join();
                    joined = true;
                    ScfOutput out = d.run(bases[i], setup, m.scf, m.n_alpha, m.n_beta, warm ? prevA.data() : nullptr,
                                          warm && nspin == 2 ? prevB.data() : nullptr, kBatchDeltaThr, m.ctl);
                    builder.leave();
                    joined = false;
                    prevA = out.P;
                    prevB = out.P2;
                    done(i, &out, out.converged ? HFX_OK : HFX_ERR_NOT_CONVERGED, std::string());
                } catch (const Error& e) {
                    if (joined) builder.leave();
                    prevA.clear();
                    prevB.clear();
                    done(i, nullptr, e.code, e.what());
                } catch (const std::exception& e) {
                    if (joined) builder.leave();
                    prevA.clear();
                    prevB.clear();
                    done(i, nullptr, HFX_ERR_CUDA, e.what());
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int w = 0; w < workers; ++w) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
    PackedRunStats st;
    st.setup_s = t_setup;
    st.builds = builder.builds();
    st.build_ms = builder.build_ms();
    st.quartets = job.stats.quartets;
    st.flops_fp64 = job.stats.flops_fp64;
    return st;
}

}  // namespace hfx

using namespace hfx;

extern "C" hfx_status hfx_batch_scf(const hfx_molecule* mols, int n, const int* n_alpha, const int* n_beta,
                                    const hfx_scf_options* scf, const hfx_batch_options* bo,
                                    hfx_scf_result* results, hfx_batch_stats* stats)
{
    try {
        if (!mols || n <= 0 || !results) throw Error(HFX_ERR_INVALID, "batch: null molecules/results or n <= 0");
        hfx_batch_options b{};
        if (bo) b = *bo;
        if (b.method != 0 && b.method != 1) throw Error(HFX_ERR_INVALID, "batch: method must be 0 (RHF) or 1 (UHF)");
        const int nspin = b.method == 1 ? 2 : 1;
        if (nspin == 2 && (!n_alpha || !n_beta)) throw Error(HFX_ERR_INVALID, "batch UHF: n_alpha/n_beta required");
        hfx_scf_options o{};
        if (scf) o = *scf;
        const double t0 = now_s();
        std::vector<Basis> bases;
        bases.reserve(n);
        for (int i = 0; i < n; ++i) bases.push_back(build_basis(mols[i]));
        hfx_options jo{};
        jo.screening_threshold = o.screening_threshold;
        jo.precision = o.precision;
        jo.fp32_threshold = o.fp32_threshold;
        std::vector<PackedMember> members(n);
        if (b.warm_chain < 0) throw Error(HFX_ERR_INVALID, "batch: warm_chain must be >= 0");
        for (int i = 0; i < n; ++i) {
            members[i].scf = o;
            members[i].n_alpha = nspin == 2 ? n_alpha[i] : 0;
            members[i].n_beta = nspin == 2 ? n_beta[i] : 0;
            members[i].warm_from = (b.warm_chain > 1 && i % b.warm_chain != 0) ? i - 1 : -1;
        }
        std::vector<hfx_status> status(n, HFX_OK);
        std::vector<std::string> msg(n);
        const PackedRunStats rs =
            run_packed(bases, jo, nspin, members, b.max_parallel,
                       [&](int i, ScfOutput* out, hfx_status st, const std::string& m) {
                           if (out)
                               fill(*out, &results[i]);
                           else
                               std::memset(&results[i], 0, sizeof(results[i]));
                           status[i] = st;
                           msg[i] = m;
                       });
        if (stats) {
            std::memset(stats, 0, sizeof(*stats));
            stats->seconds = now_s() - t0;
            stats->setup_seconds = rs.setup_s;
            stats->cycles = rs.builds;
            stats->molecules = n;
            stats->build_ms = rs.build_ms;
            stats->quartets = rs.quartets;
            stats->flops_fp64 = rs.flops_fp64;
        }
        hfx_status worst = HFX_OK;
        for (int i = 0; i < n; ++i) {
            if (status[i] != HFX_OK && status[i] != HFX_ERR_NOT_CONVERGED) {
                set_last_error("molecule " + std::to_string(i) + ": " + msg[i]);
                return status[i];
            }
            if (status[i] == HFX_ERR_NOT_CONVERGED) worst = HFX_ERR_NOT_CONVERGED;
        }
        if (worst != HFX_OK) set_last_error("batch: some molecules did not converge within max_iterations");
        return worst;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return HFX_ERR_CUDA;
    }
}
