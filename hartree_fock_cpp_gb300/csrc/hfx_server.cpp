// hfx_server.cpp -- the request server: continuous batching of RHF/UHF jobs
// on one GPU.
//
// The reference's only multi-job drivers run SCFs one after another
// (run_bl_scan, run.hpp:300-423; run_dissociation, run.hpp:498-577).  Here a
// pool of worker threads pulls requests from a queue as they arrive; a request
// is admitted when a worker slot is free and its estimated HBM footprint fits
// the remaining budget.  Every admitted job keeps its own device-resident
// state (basis, pair data, Schwarz table, quartet lists, density, DIIS
// history) and its own CUDA streams, so the Fock-build kernels of all running
// jobs are in flight on the device together and each job's host-side DIIS
// step overlaps the others' GPU work.  Jobs finish, free their slot and
// budget, and queued requests are admitted in their place.
//
// Packed mode (pack_max > 1): every admitted request still builds its own
// job on its worker, then joins a Fock session (hfx_session.cpp) shared with
// the running requests of the same method, options and size class: from its
// next SCF cycle on, its quartets are part of the session's launches -- one
// launch per quartet class per cycle over all members.  A request that
// arrives while others iterate is admitted as soon as a worker slot and
// memory are free and enters the running builds; each member leaves when
// its own SCF ends (at most pack_max members per session).
//
// Failures stay with the job that caused them: a bad basis file, an
// unsupported element, a footprint above the whole budget, an allocation
// failure, a cancellation or a timeout ends that job with its status code.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "hfx_batch.hpp"
#include "hfx_dscf.hpp"
#include "hfx_engine.hpp"
#include "hfx_scf.hpp"
#include "hfx_session.hpp"

namespace hfx {

static double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct ServerJob {
    long long id = 0;
    // owned copy of the request
    std::vector<std::string> symbols;
    std::vector<double> xyz;
    std::string basis_set, basis_path;
    int method = 0;
    int n_alpha = 0, n_beta = 0;
    hfx_scf_options scf{};
    int precision = 0;
    double fp32_threshold = 0.0;
    double timeout_s = 0.0;
    int inject_fault = 0;
    std::vector<double> P0a, P0b;
    // state
    int state = HFX_JOB_QUEUED;
    hfx_status status = HFX_OK;
    std::string message;
    double t_submit = 0, t_admit = 0, t_end = 0;
    double E_tot = 0, fock_ms = 0;
    int iterations = 0, converged = 0, K = 0, fock_builds = 0;
    size_t footprint = 0;
    std::vector<double> Pa, Pb;
    std::atomic<bool> cancel{false};
};

// A server job's view of its Fock session, as the device SCF sees a builder.
class SessionMember final : public FockSource {
public:
    explicit SessionMember(const Job& job) : K_(job.K()), mixed_(job.mixed())
    {
        cuda_check(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking), "cudaStreamCreate");
    }
    ~SessionMember() override
    {
        if (st_) {
            cudaStreamSynchronize(st_);
            cudaStreamDestroy(st_);
        }
    }
    void attach(FockSession* s, int slot)
    {
        s_ = s;
        slot_ = slot;
    }
    int K() const override { return K_; }
    cudaStream_t stream() const override { return st_; }
    bool mixed() const override { return mixed_; }
    void fock_rhf_device_ex(const double* dP, double* dG, bool mixed, double dthr) override
    {
        s_->build(slot_, st_, dP, nullptr, dG, nullptr, nullptr, mixed, dthr, &ms_);
    }
    void fock_uhf_device_ex(const double* dPa, const double* dPb, double* dJ, double* dKa, double* dKb, bool mixed,
                            double dthr) override
    {
        s_->build(slot_, st_, dPa, dPb, dJ, dKa, dKb, mixed, dthr, &ms_);
    }
    double last_build_ms() const override { return ms_; }

private:
    FockSession* s_ = nullptr;
    int slot_ = -1;
    int K_;
    bool mixed_;
    cudaStream_t st_ = nullptr;
    double ms_ = 0.0;
};

class Server {
public:
    explicit Server(const hfx_server_options& o) : opt_(o)
    {
        if (opt_.max_active <= 0) opt_.max_active = 8;
        cuda_check(cudaSetDevice(opt_.device), "cudaSetDevice");
        size_t free_b = 0, total_b = 0;
        cuda_check(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
        budget_ = opt_.hbm_budget_gb > 0 ? (size_t)(opt_.hbm_budget_gb * 1e9) : (size_t)(0.8 * free_b);
        for (int w = 0; w < opt_.max_active; ++w) workers_.emplace_back([this] { worker(); });
    }

    ~Server()
    {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
            for (auto& kv : jobs_) kv.second->cancel = true;
        }
        cv_.notify_all();
        for (auto& t : workers_) t.join();
    }

    long long submit(const hfx_request& r)
    {
        if (!r.mol.symbols || !r.mol.xyz || !r.mol.basis_set || r.mol.natom <= 0)
            throw Error(HFX_ERR_INVALID, "request: molecule incomplete");
        auto j = std::make_shared<ServerJob>();
        for (int a = 0; a < r.mol.natom; ++a) j->symbols.emplace_back(r.mol.symbols[a]);
        j->xyz.assign(r.mol.xyz, r.mol.xyz + 3 * r.mol.natom);
        j->basis_set = r.mol.basis_set;
        if (r.mol.basis_path) j->basis_path = r.mol.basis_path;
        j->method = r.method;
        j->n_alpha = r.n_alpha;
        j->n_beta = r.n_beta;
        j->scf = r.scf;
        j->precision = r.precision < 0 ? opt_.precision : r.precision;
        j->fp32_threshold = r.fp32_threshold > 0 ? r.fp32_threshold : opt_.fp32_threshold;
        // the SCF follows the job's precision: a mixed-precision job runs the
        // mixed-precision protocol (FP32 builds, then FP64 final cycles)
        j->scf.precision = j->precision;
        j->scf.fp32_threshold = j->fp32_threshold;
        j->timeout_s = r.timeout_s;
        j->inject_fault = r.inject_fault;
        j->t_submit = now_s();
        std::lock_guard<std::mutex> lk(mu_);
        j->id = next_id_++;
        jobs_[j->id] = j;
        queue_.push_back(j);
        cv_.notify_one();
        return j->id;
    }

    void info(long long id, hfx_job_info* out)
    {
        std::lock_guard<std::mutex> lk(mu_);
        auto it = jobs_.find(id);
        if (it == jobs_.end()) throw Error(HFX_ERR_INVALID, "unknown job id");
        fill(*it->second, out);
    }

    bool wait(long long id, double timeout_s, hfx_job_info* out)
    {
        std::unique_lock<std::mutex> lk(mu_);
        auto it = jobs_.find(id);
        if (it == jobs_.end()) throw Error(HFX_ERR_INVALID, "unknown job id");
        auto j = it->second;
        auto pred = [&] { return j->state == HFX_JOB_DONE || j->state == HFX_JOB_FAILED; };
        bool ok = timeout_s > 0 ? done_cv_.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)
                                : (done_cv_.wait(lk, pred), true);
        if (out) fill(*j, out);
        return ok;
    }

    void cancel(long long id)
    {
        std::lock_guard<std::mutex> lk(mu_);
        auto it = jobs_.find(id);
        if (it == jobs_.end()) throw Error(HFX_ERR_INVALID, "unknown job id");
        it->second->cancel = true;
        cv_.notify_all();
    }

    bool drain(double timeout_s)
    {
        std::unique_lock<std::mutex> lk(mu_);
        auto pred = [&] { return queue_.empty() && running_ == 0; };
        if (timeout_s > 0) return done_cv_.wait_for(lk, std::chrono::duration<double>(timeout_s), pred);
        done_cv_.wait(lk, pred);
        return true;
    }

    void density(long long id, double* Pa, double* Pb)
    {
        std::lock_guard<std::mutex> lk(mu_);
        auto it = jobs_.find(id);
        if (it == jobs_.end()) throw Error(HFX_ERR_INVALID, "unknown job id");
        const auto& j = *it->second;
        if (j.state != HFX_JOB_DONE) throw Error(HFX_ERR_INVALID, "job has no result");
        if (Pa && !j.Pa.empty()) std::memcpy(Pa, j.Pa.data(), j.Pa.size() * sizeof(double));
        if (Pb && !j.Pb.empty()) std::memcpy(Pb, j.Pb.data(), j.Pb.size() * sizeof(double));
    }

    void stats(hfx_server_stats_t* s)
    {
        std::lock_guard<std::mutex> lk(mu_);
        std::memset(s, 0, sizeof(*s));
        s->queued = (int)queue_.size();
        s->running = running_;
        s->budget_bytes = (double)budget_;
        s->in_use_bytes = (double)in_use_;
        s->max_concurrent = max_concurrent_;
        s->max_session_members = max_session_members_;
        s->sessions_created = sessions_created_;
        for (auto& kv : jobs_) {
            if (kv.second->state == HFX_JOB_DONE) ++s->done;
            if (kv.second->state == HFX_JOB_FAILED) ++s->failed;
        }
    }

private:
    static void fill(const ServerJob& j, hfx_job_info* o)
    {
        std::memset(o, 0, sizeof(*o));
        o->state = j.state;
        o->status = j.status;
        o->E_tot = j.E_tot;
        o->iterations = j.iterations;
        o->converged = j.converged;
        o->K = j.K;
        o->t_submit = j.t_submit;
        o->t_admit = j.t_admit;
        o->t_end = j.t_end;
        o->fock_ms = j.fock_ms;
        o->fock_builds = j.fock_builds;
        std::strncpy(o->message, j.message.c_str(), sizeof(o->message) - 1);
    }

    // device bytes a job will hold: pair data and records, quartet lists,
    // J/K and SCF work matrices
    static size_t estimate_footprint(const Basis& b)
    {
        size_t K = b.K, prims = 0, pairs = 0;
        for (size_t x = 0; x < b.shells.size(); ++x)
            for (size_t y = 0; y <= x; ++y) {
                ++pairs;
                prims += (size_t)b.shells[x].nprim() * b.shells[y].nprim();
            }
        const size_t per_prim_pair = 8 * (4 + 100) * 2 + 8 * 36 * 35;    // records (64+32 bit) + dense E bound
        const size_t tasks = pairs * pairs / 2 * 12 / 4;                  // screened list, generous
        return prims * per_prim_pair + tasks + 8 * K * K * 64 + (size_t(64) << 20);
    }

    void worker()
    {
        cudaSetDevice(opt_.device);
        while (true) {
            std::shared_ptr<ServerJob> j;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return stop_ || !queue_.empty(); });
                if (stop_) return;
                // admission: first queued job whose footprint fits (cancelled ones drop out)
                for (auto it = queue_.begin(); it != queue_.end(); ++it) {
                    auto& c = *it;
                    if (c->cancel) {
                        c->state = HFX_JOB_FAILED;
                        c->status = HFX_ERR_CANCELLED;
                        c->message = "cancelled before admission";
                        c->t_end = now_s();
                        queue_.erase(it);
                        done_cv_.notify_all();
                        j = nullptr;
                        break;
                    }
                    j = c;
                    queue_.erase(it);
                    break;
                }
                if (!j) continue;
                ++running_;
                j->state = HFX_JOB_RUNNING;
                j->t_admit = now_s();
                max_concurrent_ = std::max(max_concurrent_, running_);
            }
            run(j);
            {
                std::lock_guard<std::mutex> lk(mu_);
                --running_;
                in_use_ -= j->footprint;
                j->t_end = now_s();
            }
            done_cv_.notify_all();
            cv_.notify_all();
        }
    }

    // reserve the job's footprint, waiting (bounded by the job's timeout) for
    // running jobs to release memory; a footprint above the whole budget fails
    void reserve(ServerJob& j, size_t bytes)
    {
        std::unique_lock<std::mutex> lk(mu_);
        if (bytes > budget_) throw Error(HFX_ERR_OOM, "estimated device footprint exceeds the server's HBM budget");
        const double t0 = now_s();
        while (in_use_ + bytes > budget_) {
            if (j.cancel) throw Error(HFX_ERR_CANCELLED, "cancelled while waiting for memory");
            if (j.timeout_s > 0 && now_s() - j.t_submit > j.timeout_s)
                throw Error(HFX_ERR_TIMEOUT, "timed out waiting for device memory");
            done_cv_.wait_for(lk, std::chrono::milliseconds(20));
            if (now_s() - t0 > 3600.0) throw Error(HFX_ERR_TIMEOUT, "admission wait exceeded one hour");
        }
        in_use_ += bytes;
        j.footprint = bytes;
    }

    // Size class of a job for session grouping: a small job does not wait
    // each cycle on the O(K^3) steps of a large one.
    static int size_class(int K) { return K < 100 ? 0 : (K < 300 ? 1 : 2); }

    // The session a packed-mode job joins: one with the same method, options
    // and size class that has room, else a new one.  Joining happens under
    // the server lock, so a session found here is not dropped meanwhile.
    std::shared_ptr<FockSession> join_session(const ServerJob& j, Job& job, int nspin, int* slot)
    {
        std::lock_guard<std::mutex> lk(mu_);
        auto key = std::make_tuple(j.method, j.precision, j.fp32_threshold, job.screening_threshold(),
                                   size_class(job.K()));
        auto& list = sessions_[key];
        for (auto& s : list)
            if (!s->failed() && s->members() < opt_.pack_max) {
                *slot = s->join(job);
                max_session_members_ = std::max(max_session_members_, s->members());
                return s;
            }
        auto s = std::make_shared<FockSession>(opt_.device, nspin, job.screening_threshold());
        *slot = s->join(job);
        list.push_back(s);
        ++sessions_created_;
        max_session_members_ = std::max(max_session_members_, 1);
        return s;
    }

    // A member's SCF ended: leave, and drop the session once it is empty
    // (a job that joined it meanwhile keeps it alive through its own handle).
    void leave_session(const std::shared_ptr<FockSession>& s, int slot)
    {
        s->leave(slot);
        std::lock_guard<std::mutex> lk(mu_);
        if (s->members() > 0) return;
        for (auto& kv : sessions_) {
            auto& list = kv.second;
            list.erase(std::remove(list.begin(), list.end(), s), list.end());
        }
    }

    void run(std::shared_ptr<ServerJob> j)
    {
        try {
            if (j->inject_fault == HFX_FAULT_SETUP) throw Error(HFX_ERR_INVALID, "injected fault during setup");
            std::vector<const char*> syms;
            for (auto& s : j->symbols) syms.push_back(s.c_str());
            hfx_molecule mol{(int)syms.size(), syms.data(), j->xyz.data(), j->basis_set.c_str(),
                             j->basis_path.empty() ? nullptr : j->basis_path.c_str()};
            Basis b = build_basis(mol);
            j->K = b.K;
            size_t fp = estimate_footprint(b);
            if (j->inject_fault == HFX_FAULT_OOM) fp = budget_ + 1;
            reserve(*j, fp);
            if (j->inject_fault == HFX_FAULT_ALLOC) throw Error(HFX_ERR_OOM, "injected allocation failure");
            hfx_options o{};
            o.screening_threshold = j->scf.screening_threshold;
            o.precision = j->precision;
            o.fp32_threshold = j->fp32_threshold;
            o.device = opt_.device;
            Job job(b, o);
            ScfSetup setup = scf_setup(b, true);
            const int nspin = j->method == 1 ? 2 : 1;
            const double deadline = j->timeout_s > 0 ? j->t_submit + j->timeout_s : 0.0;
            ScfControl ctl{&j->cancel, deadline, j->inject_fault == HFX_FAULT_ITERATION ? 3 : 0};
            ScfOutput out;
            if (opt_.pack_max > 1) {
                // packed mode: the job's builds run inside a shared Fock session
                SessionMember member(job);
                DeviceScf d(member, setup, nspin);
                int slot = -1;
                std::shared_ptr<FockSession> sess = join_session(*j, job, nspin, &slot);
                member.attach(sess.get(), slot);
                try {
                    out = d.run(b, setup, j->scf, j->n_alpha, j->n_beta, nullptr, nullptr, 1e-12, &ctl);
                } catch (...) {
                    leave_session(sess, slot);
                    throw;
                }
                leave_session(sess, slot);
            } else {
                DeviceScf d(job, setup, nspin);
                out = d.run(b, setup, j->scf, j->n_alpha, j->n_beta, nullptr, nullptr, 1e-12, &ctl);
            }
            std::lock_guard<std::mutex> lk(mu_);
            j->E_tot = out.E_tot;
            j->iterations = out.iterations;
            j->converged = out.converged;
            j->fock_ms = out.fock_ms;
            j->fock_builds = out.fock_builds;
            j->Pa = std::move(out.P);
            j->Pb = std::move(out.P2);
            j->status = out.converged ? HFX_OK : HFX_ERR_NOT_CONVERGED;
            j->state = HFX_JOB_DONE;
        } catch (const Error& e) {
            std::lock_guard<std::mutex> lk(mu_);
            j->status = e.code;
            j->message = e.what();
            j->state = HFX_JOB_FAILED;
        } catch (const std::exception& e) {
            std::lock_guard<std::mutex> lk(mu_);
            j->status = HFX_ERR_INVALID;
            j->message = e.what();
            j->state = HFX_JOB_FAILED;
        }
    }

    hfx_server_options opt_;
    size_t budget_ = 0, in_use_ = 0;
    std::mutex mu_;
    std::condition_variable cv_, done_cv_;
    std::deque<std::shared_ptr<ServerJob>> queue_;
    std::map<long long, std::shared_ptr<ServerJob>> jobs_;
    std::map<std::tuple<int, int, double, double, int>, std::vector<std::shared_ptr<FockSession>>> sessions_;
    std::vector<std::thread> workers_;
    long long next_id_ = 1;
    int running_ = 0, max_concurrent_ = 0;
    int max_session_members_ = 0, sessions_created_ = 0;
    bool stop_ = false;
};

}  // namespace hfx

struct hfx_server {
    std::unique_ptr<hfx::Server> s;
};

using namespace hfx;

template <typename F>
static hfx_status sguard(F&& f)
{
    try {
        f();
        return HFX_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return HFX_ERR_INVALID;
    }
}

extern "C" {

hfx_status hfx_server_create(const hfx_server_options* opt, hfx_server** out)
{
    return sguard([&] {
        if (!out) throw Error(HFX_ERR_INVALID, "null argument");
        hfx_server_options o{};
        if (opt) o = *opt;
        auto s = std::make_unique<hfx_server>();
        s->s = std::make_unique<Server>(o);
        *out = s.release();
    });
}

hfx_status hfx_server_submit(hfx_server* s, const hfx_request* r, long long* id)
{
    return sguard([&] {
        if (!s || !r || !id) throw Error(HFX_ERR_INVALID, "null argument");
        *id = s->s->submit(*r);
    });
}

hfx_status hfx_server_poll(hfx_server* s, long long id, hfx_job_info* info)
{
    return sguard([&] {
        if (!s || !info) throw Error(HFX_ERR_INVALID, "null argument");
        s->s->info(id, info);
    });
}

hfx_status hfx_server_wait(hfx_server* s, long long id, double timeout_s, hfx_job_info* info)
{
    return sguard([&] {
        if (!s) throw Error(HFX_ERR_INVALID, "null argument");
        if (!s->s->wait(id, timeout_s, info)) throw Error(HFX_ERR_TIMEOUT, "wait timed out");
    });
}

hfx_status hfx_server_cancel(hfx_server* s, long long id)
{
    return sguard([&] {
        if (!s) throw Error(HFX_ERR_INVALID, "null argument");
        s->s->cancel(id);
    });
}

hfx_status hfx_server_drain(hfx_server* s, double timeout_s)
{
    return sguard([&] {
        if (!s) throw Error(HFX_ERR_INVALID, "null argument");
        if (!s->s->drain(timeout_s)) throw Error(HFX_ERR_TIMEOUT, "drain timed out");
    });
}

hfx_status hfx_server_density(hfx_server* s, long long id, double* Pa, double* Pb)
{
    return sguard([&] {
        if (!s) throw Error(HFX_ERR_INVALID, "null argument");
        s->s->density(id, Pa, Pb);
    });
}

hfx_status hfx_server_stats(hfx_server* s, hfx_server_stats_t* st)
{
    return sguard([&] {
        if (!s || !st) throw Error(HFX_ERR_INVALID, "null argument");
        s->s->stats(st);
    });
}

hfx_status hfx_server_destroy(hfx_server* s)
{
    return sguard([&] { delete s; });
}

}  // extern "C"
