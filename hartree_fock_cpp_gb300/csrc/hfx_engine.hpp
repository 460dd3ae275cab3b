// hfx_engine.hpp -- the device-resident job: pair data, Schwarz tables,
// screened shell-quartet work lists, and the Fock-build entry points.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <tuple>
#include <vector>

#include "hfx_device.cuh"
#include "hfx_internal.hpp"

namespace hfx {

// device launch helpers (hfx_kernels.cu)
size_t generic_smem_bytes(int maxacc, int maxw, int maxr);
cudaError_t launch_eri(const LaunchArgs& a, int maxacc, int maxw, int maxr, int grid, cudaStream_t st);
// symmetrisation of packed accumulators: one grid row (blockIdx.y) per
// molecule, Kmax = the largest molecule's K
KernelSpec finish_rhf_spec(int Kmax, int nfrag);   // k_finish_rhf(Jacc, Kacc, G, fk, fmoff, active)
KernelSpec finish_uhf_spec(int Kmax, int nfrag);   // k_finish_uhf(Jacc, Ka, Kb, J, Kao, Kbo, fk, fmoff, active)
KernelSpec add_spec(long long n);    // k_add(A, B, C, n)
KernelSpec to_float_spec(long long n);   // k_to_float(A, B, n)
KernelSpec density_blocks_spec(int npairs);   // k_density_blocks(pairs, npairs, D1, D2, Dsh)
KernelSpec rebase_tasks_spec(long long n);    // k_rebase_tasks(tasks, n, delta): bra, ket += delta
cudaError_t small_spec_f64(int pcb, int pck, int nk, int ntasks, KernelSpec* s);   // k_small(SmallArgs<double>)
cudaError_t small_spec_f32(int pcb, int pck, int nk, int ntasks, KernelSpec* s);   // k_small(SmallArgs<float>)
cudaError_t warp_spec(bool fp32, int nk, int grid, int warps_per_cta, int slice, KernelSpec* s);
cudaError_t launch_warp(bool fp32, const void* args, int nk, int grid, int warps_per_cta, cudaStream_t st);
// shared-memory slice (elements) of a warp task; the lane-parallel R mode (L <= 6,
// ket npp >= lane_min_npp, 0: never) needs 32 R vectors, the level-parallel one a round
int warp_slice_elems(int l0b, int l1b, int l0k, int l1k, int npp_ket, int lane_min_npp);
constexpr int kDefaultLaneMinNpp = 6;
bool is_small_class(int pcb, int pck);
// Boys table of the kernels ([kBoysN][kBoysM], last column exp(-T_k)), built once per process.
const std::vector<double>& boys_table_host();
// The FP32 kernels' Boys table: 8 floats per (L <= kBoys32MaxL, k), see hfx_device.cuh.
const std::vector<float>& boys_table32_host();
// The FP64 Fock kernels' Boys table: 8 doubles per (L <= kBoys64MaxL, k), see hfx_device.cuh.
const std::vector<double>& boys_table64_host();

void cuda_check(cudaError_t e, const char* what);

// Caching device allocator: freed blocks (rounded up to a power of two, up to
// 256 MB) are kept for reuse instead of being returned with cudaFree, whose
// implicit device synchronisation would stall every other job in flight when
// one job of the request server finishes.  Larger blocks are allocated and
// freed directly.  Callers free a block only after the work using it has
// completed (a job synchronises its streams before its buffers go).
void* pool_alloc(size_t bytes);
void pool_free(void* p, size_t bytes);
size_t pool_cached_bytes();

// Owning device buffer.
template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { reset(); }
    void reset()
    {
        if (p) pool_free(p, n * sizeof(T));
        p = nullptr;
        n = 0;
    }
    void alloc(size_t count)
    {
        if (count == n && p) return;
        reset();
        if (count == 0) return;
        p = static_cast<T*>(pool_alloc(count * sizeof(T)));
        n = count;
    }
    void upload(const std::vector<T>& v, cudaStream_t st)
    {
        alloc(v.size());
        if (!v.empty()) cuda_check(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st), "upload");
    }
};

struct HostPair {
    int frag;         // molecule of a packed job
    int s0, s1;       // shells (s0 has the higher L), indices in the concatenated basis
    int l0, l1;
    int npp;
    long long e_off;
    int pp0;
    bool same;
};

// Host image of the per-job pair data (built on the CPU, then uploaded).
struct PairData {
    std::vector<HostPair> hpairs;
    std::vector<DPair> dpairs;
    std::vector<PairGeo> geo;
    std::vector<double> epool;
    std::vector<double> rec;   // class-kernel primitive-pair records
};

// Per pair class: component-pair / coefficient layout of the records.
struct ClassTables {
    std::vector<PairClassTab> tab;
    std::vector<int> ab_start;
    std::vector<short> k_herm, k_lin;
};
const ClassTables& class_tables();

// One kernel launch of a Fock build.
struct LaunchGroup {
    int kind;            // 0: small-class kernel, 1: warp kernel
    int pcb, pck;        // small-class kernel class
    bool fp32;
    int slice;           // warp kernel: per-warp slice (elements)
    int warps_per_cta;
    int lane_min_npp;    // warp kernel: lane-parallel R threshold the slice was sized for
    int grid;
    size_t off, n;       // task range in the concatenated list
    double flops, prims;
};
// Molecules of a packed job (one entry for a plain job): molecule f owns
// shells [sh[f], sh[f+1]) and basis functions [bf[f], bf[f+1]) of the
// concatenated basis, shell pairs [pbase[f], pbase[f+1]), the K_f x K_f
// block at moff[f] of every packed matrix buffer and the BF-pair bounds at
// qoff[f].
struct Fragments {
    std::vector<int> sh, bf, pbase;
    std::vector<long long> moff, qoff;
    int count() const { return (int)sh.size() - 1; }
    int K(int f) const { return bf[f + 1] - bf[f]; }
    long long nmat() const { return moff.back(); }
};
// Concatenate molecules' bases (shell bf0 shifted to the concatenated order)
// and describe the blocks.
Basis concat_basis(const std::vector<Basis>& mols, Fragments& fr);
Fragments single_fragment(const Basis& b);

PairData build_pair_data(const Basis& b, const Fragments& fr);

// The launch plan of one precision mode.
struct GroupSet {
    std::vector<LaunchGroup> groups;
    DevBuf<Task> tasks;
    int ntasks = 0, nquartets = 0;
    double flops64 = 0.0, flops32 = 0.0, prims = 0.0, quartets32 = 0.0;
};

// Destination of a Fock build's device work.  Lane 0 is the job's main
// stream, lanes 1..n its auxiliary streams; fork() makes every auxiliary lane
// wait for what lane 0 has issued so far, join() makes lane 0 wait for all of
// them.  StreamSink issues the work on the streams as it comes; GraphSink
// records it as the nodes and edges of a CUDA graph, built node by node
// rather than by stream capture, so other threads' CUDA calls (allocations,
// module loads, library handles of concurrent jobs) cannot invalidate it.
class OpSink {
public:
    virtual ~OpSink() = default;
    virtual void zero(int lane, void* p, size_t bytes) = 0;
    virtual void kernel(int lane, const KernelSpec& s, void** params) = 0;
    virtual void fork() = 0;
    virtual void join() = 0;
};

class StreamSink final : public OpSink {
public:
    StreamSink(cudaStream_t main, const std::vector<cudaStream_t>& aux, cudaEvent_t fork_ev,
               const std::vector<cudaEvent_t>& aux_ev);
    void zero(int lane, void* p, size_t bytes) override;
    void kernel(int lane, const KernelSpec& s, void** params) override;
    void fork() override;
    void join() override;

private:
    cudaStream_t stream(int lane) const { return lane == 0 ? main_ : aux_[lane - 1]; }
    cudaStream_t main_;
    const std::vector<cudaStream_t>& aux_;
    cudaEvent_t fork_ev_;
    const std::vector<cudaEvent_t>& aux_ev_;
};

class GraphSink final : public OpSink {
public:
    explicit GraphSink(int lanes);
    ~GraphSink() override;
    void zero(int lane, void* p, size_t bytes) override;
    void kernel(int lane, const KernelSpec& s, void** params) override;
    void fork() override;
    void join() override;
    cudaGraphExec_t instantiate();

private:
    cudaGraph_t graph_ = nullptr;
    std::vector<std::vector<cudaGraphNode_t>> deps_;   // per lane: the nodes its next node depends on
};

// What the device SCF needs from a Fock builder: a job of its own, or one
// molecule's share of a packed job (hfx_batch.cpp).  Builds are synchronous
// with respect to stream().
class FockSource {
public:
    virtual ~FockSource() = default;
    virtual int K() const = 0;
    virtual cudaStream_t stream() const = 0;
    virtual bool mixed() const = 0;
    virtual void fock_rhf_device_ex(const double* dP, double* dG, bool mixed, double dthr) = 0;
    virtual void fock_uhf_device_ex(const double* dPa, const double* dPb, double* dJ, double* dKa, double* dKb,
                                    bool mixed, double dthr) = 0;
    virtual double last_build_ms() const = 0;   // device time of the last build
};

class FockSession;

class Job final : public FockSource {
    friend class FockSession;   // reads the device pair tables and plans of its members

public:
    Job(Basis b, const hfx_options& opt);
    // Packed job over several molecules: shell pairs and quartets never mix
    // molecules, and every Fock build works on packed buffers holding each
    // molecule's K_f x K_f matrices back to back (the blocks of fragments()).
    Job(const std::vector<Basis>& mols, const hfx_options& opt);
    ~Job();

    const Fragments& fragments() const { return frags_; }
    long long nmat() const { return frags_.nmat(); }
    // packed jobs: molecules whose flag is 0 are skipped by the next builds
    void set_active(const unsigned char* flags);

    int K() const override { return basis_.K; }
    int device() const { return device_; }
    const Basis& basis() const { return basis_; }

    void schwarz_host(std::vector<double>& Qbf) const;
    // device-pointer Fock builds (synchronous)
    void fock_rhf_device(const double* dP, double* dG);
    // Builds with an explicit precision plan (mixed = false: every quartet in
    // FP64) and density-weighted screening threshold (0: none; used by the
    // incremental builds of the mixed-precision SCF).
    void fock_rhf_device_ex(const double* dP, double* dG, bool mixed, double dthr) override;
    void fock_uhf_device_ex(const double* dPa, const double* dPb, double* dJ, double* dKa, double* dKb, bool mixed,
                            double dthr) override;
    double last_build_ms() const override { return stats.ms; }
    void fock_rhf_ex(const double* P, double* G, bool mixed, double dthr);
    void fock_uhf_ex(const double* Pa, const double* Pb, double* J, double* Ka, double* Kb, bool mixed, double dthr);
    bool mixed() const override { return opt_.precision == HFX_PREC_MIXED; }
    double fp32_threshold() const { return opt_.fp32_threshold; }
    double screening_threshold() const { return opt_.screening_threshold; }
    // Pick the FP32 threshold: for each candidate (largest first) build G in
    // mixed precision at density P and keep the largest tau whose energy
    // change 1/2 sum P (G_tau - G_fp64) stays within target_dE; the job is
    // switched to mixed precision at that tau.  Returns tau (0 if none fits).
    double autotune_fp32_threshold(const double* P, double target_dE, double* dE_out, double* ms_fp64,
                                   double* ms_mixed);
    // RHF build whose scratch (J/K accumulators, work-queue counters) is
    // supplied by the caller; allocates nothing.  Jacc/Kacc hold K*K doubles,
    // counters num_launch_groups() ints.
    void fock_rhf_device_scratch(const double* dP, double* dG, double* Jacc, double* Kacc, int* counters);
    // launch shape of the plans (chunk sizes, warps per CTA); setting it rebuilds the plans
    const hfx_launch_shape& launch_shape() const { return shape_; }
    void set_launch_shape(const hfx_launch_shape& s);
    // pick the launch shape by timing builds at density P (host, K x K); returns the best build ms
    double autotune_launch_shape(const double* P, int builds, hfx_launch_shape* out);
    int num_launch_groups() const { return (int)plan(true).groups.size(); }
    // launch groups of a plan (FP64 or, for a mixed job, mixed)
    const std::vector<LaunchGroup>& plan_groups(bool mixed_plan) const { return plan(mixed_plan).groups; }
    void fock_uhf_device(const double* dPa, const double* dPb, double* dJ, double* dKa, double* dKb);
    void fock_rhf(const double* P, double* G);
    void fock_uhf(const double* Pa, const double* Pb, double* J, double* Ka, double* Kb);
    void eri_unique(double thr, double* out);

    hfx_build_stats stats{};
    cudaStream_t stream() const override { return stream_; }

private:
    void init(const hfx_options& opt);
    void build_pairs();
    void compute_schwarz();
    void build_tasks(double thr, std::vector<Task>& tasks, int& maxacc, int& maxw, int& maxr, double* flops = nullptr,
                     double* prims = nullptr) const;
    void run_eri_tasks(const DevBuf<Task>& tasks, int ntasks, int maxacc, int maxw, int maxr, LaunchArgs a);
    LaunchArgs base_args() const;
    template <typename F>
    void for_each_surviving_quartet(double thr, F&& f) const;
    void record_stats(int launches);

    Basis basis_;
    hfx_options opt_;
    int device_ = 0;
    int nsm_ = 1;
    cudaStream_t stream_ = nullptr;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr, evk0_ = nullptr, evk1_ = nullptr;

    void build_jk_groups(bool mixed, GroupSet& gs);
    void launch_jk(OpSink& sk, int nk, const double* Dj, const double* Dk, const double* Dk2, double* J, double* Kx,
                   double* Kx2, int* counters = nullptr, bool mixed_plan = false, double dthr = 0.0);
    const GroupSet& plan(bool mixed_plan) const { return mixed_plan && mixed() ? gs_mixed_ : gs_fp64_; }
    void record_stats_plan(int launches, const GroupSet& gs);
    StreamSink stream_sink() { return StreamSink(stream_, aux_, fork_ev_, aux_ev_); }
    int max_fragment_K() const;
    void enqueue_finish_rhf(OpSink& sk, const double* Jacc, const double* Kacc, double* dG);
    void enqueue_rhf(OpSink& sk, const double* dP, double* dG, bool mixed_plan, double dthr);
    void enqueue_uhf(OpSink& sk, const double* dPa, const double* dPb, double* dJ, double* dKa, double* dKb, bool mixed_plan,
                     double dthr);
    cudaGraphExec_t graph_for(int nk, bool mixed_plan, double dthr);
    void clear_graphs();
    struct GraphEntry {
        cudaGraphExec_t exec = nullptr;
        int eager_runs = 0;
    };
    std::map<std::tuple<int, bool, double>, GraphEntry> graphs_;
    bool no_graphs_ = false;
    DevBuf<double> d_gin_, d_gin2_, d_gout_, d_gout2_, d_gout3_;
    Fragments frags_;
    DevBuf<int> d_fk_;              // per molecule K_f
    DevBuf<long long> d_fmoff_;     // per molecule matrix offset
    DevBuf<unsigned char> d_active_;   // packed jobs: per molecule build flag
    bool packed_ = false;              // built by the packed (several-molecule) constructor
    hfx_launch_shape shape_{256, 4096, 8, kDefaultLaneMinNpp, {0, 0, 0, 0}};

    std::vector<HostPair> hpairs_;
    GroupSet gs_fp64_, gs_mixed_;
    DevBuf<int> d_counters_;
    DevBuf<double> d_dsh_;
    DevBuf<float> d_d32_;           // float copies of the build's densities (FP32 groups)
    std::vector<DPair> dpairs_host_;
    DevBuf<double> d_rec64_;
    DevBuf<float> d_rec32_;
    DevBuf<float> d_boys32_;
    DevBuf<PairClassTab> d_pct_;
    DevBuf<int> d_abs_;
    DevBuf<short> d_kh_, d_kl_;
    std::vector<cudaStream_t> aux_;
    std::vector<cudaEvent_t> aux_ev_;
    cudaEvent_t fork_ev_ = nullptr;
    double flops32_ = 0.0, quartets32_ = 0.0;
    std::vector<double> qsh_;     // per pair
    std::vector<double> qbf_;     // per BF pair
    DevBuf<DPair> d_pairs_;
    DevBuf<PairGeo> d_ppgeo_;
    DevBuf<double> d_epool_;
    DevBuf<double> d_boys_;     // [kBoysN][kBoysM] (k_quartet_eri)
    DevBuf<double> d_boys64_;   // per-L rows (FP64 Fock and Schwarz kernels)
    DevBuf<double> d_qbf_;
    DevBuf<float> d_qbf32_;         // float copy of d_qbf_ (the FP32 kernels' screen)
    DevBuf<unsigned long long> d_qsh_;
    DevBuf<Task> d_tasks_;
    int ntasks_ = 0;
    int nquartets_ = 0;
    int maxacc_ = 0, maxw_ = 0, maxr_ = 0;
    DevBuf<int> d_counter_;
    DevBuf<double> d_D_, d_D2_, d_Dj_, d_J_, d_K_, d_K2_, d_out1_, d_out2_, d_out3_;
    double prim_quartets_ = 0.0, flops_ = 0.0;
};

}  // namespace hfx
