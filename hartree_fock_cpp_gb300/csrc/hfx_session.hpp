// hfx_session.hpp -- one Fock build per SCF cycle over several independent
// jobs that join and leave while the others iterate (hfx_session.cpp).
#pragma once

#include <condition_variable>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "hfx_engine.hpp"

namespace hfx {

// A Fock session serves the request server's packed mode.  Every member is a
// complete job of its own (basis, pair records, Schwarz table, launch plans
// on the device), created by the request's worker before it joins.  Each SCF
// cycle the members rendezvous and the last to arrive runs ONE build for all
// of them: one launch per quartet class over every member's quartets (the
// members' task lists concatenated, their pair records addressed through a
// combined pair table), one density staging and one result copy per member.
// A member joins at the next cycle after its setup and leaves when its own
// SCF ends, so requests that arrive while others iterate enter the running
// builds.  Members of one session share the method (RHF / UHF) and the
// screening threshold; mixed-precision and FP64 (incremental) builds of one
// cycle run as separate variants, each with only its members switched on.
class FockSession {
public:
    FockSession(int device, int nspin, double screening_threshold);
    ~FockSession();
    FockSession(const FockSession&) = delete;
    FockSession& operator=(const FockSession&) = delete;

    // Adds a job (it must outlive its membership and have been built with
    // this session's screening threshold); returns its slot.  The job takes
    // part from the next cycle on.
    int join(Job& job);
    // Removes a member (its SCF ended or failed); never blocks on a build.
    void leave(int slot);
    // One member's build of the current cycle: the member's densities (K x K,
    // device, complete on stream st), its outputs (G, or J / Ka / Kb for
    // UHF), the precision plan and density-screening threshold.  Blocks
    // until the cycle's builds are done; *ms gets their device time.
    void build(int slot, cudaStream_t st, const double* dPa, const double* dPb, double* o0, double* o1, double* o2,
               bool mixed, double dthr, double* ms);

    int nspin() const { return nspin_; }
    int members() const;                  // live members
    int builds() const { return builds_; }
    double build_ms() const { return build_ms_; }
    int max_members() const { return max_members_; }
    bool failed() const
    {
        std::lock_guard<std::mutex> lk(mu_);
        return failed_;
    }

private:
    struct Member {
        Job* job = nullptr;
        bool live = false;
        long long moff = 0;   // first element of its matrices in the session buffers
        int pair_off = 0;     // first combined pair
        int frag = 0;         // index in the live list (active flags, finish tables)
    };
    struct Req {
        int slot;
        const double *Pa, *Pb;
        double *o0, *o1, *o2;
        bool mixed;
        double dthr;
    };
    struct Combined {
        std::vector<LaunchGroup> groups;
        DevBuf<Task> tasks;
    };

    void relayout();                      // combined tables of the live members (mu_ held)
    void combine(bool mixed_plan, Combined& c);
    void run_locked();
    void launch(int nk, bool mixed_plan, double dthr);

    int device_, nspin_, nsm_ = 1;
    double thr_;
    cudaStream_t stream_ = nullptr;
    std::vector<cudaStream_t> aux_;
    std::vector<cudaEvent_t> aux_ev_;
    cudaEvent_t fork_ev_ = nullptr, ev0_ = nullptr, ev1_ = nullptr;

    std::vector<Member> slots_;
    std::vector<int> live_;               // live slots in layout order
    bool dirty_ = true;
    long long nmat_ = 0;
    int npairs_ = 0;
    int lane_min_npp_ = kDefaultLaneMinNpp;

    // anchors of the combined pair table's offsets: each member's record and
    // Schwarz arrays are addressed as anchor + offset (one address space)
    DevBuf<double> anchor64_;
    DevBuf<float> anchor32_;
    DevBuf<DPair> pairs64_, pairs32_;
    DevBuf<int> fk_;
    DevBuf<long long> fmoff_;
    DevBuf<unsigned char> active_;
    Combined plan64_, plan_mixed_;
    DevBuf<int> counters_;
    DevBuf<double> boys64_;
    DevBuf<float> boys32_;
    DevBuf<PairClassTab> pct_;
    DevBuf<int> abs_;
    DevBuf<short> kh_, kl_;
    DevBuf<double> in_[2], dj_, acc_[3], out_[3], dsh_;
    DevBuf<float> d32_;

    mutable std::mutex mu_;
    std::condition_variable cv_;
    std::vector<Req> pending_;
    unsigned long long generation_ = 0;
    bool failed_ = false;
    hfx_status fail_code_ = HFX_OK;
    std::string fail_msg_;
    double cycle_ms_ = 0.0, build_ms_ = 0.0;
    int builds_ = 0, max_members_ = 0;
};

}  // namespace hfx
