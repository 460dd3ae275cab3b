// hfx_engine.cpp -- host side of the device-resident job.
//
// Job creation replaces what the reference does per SCF inside ERI_GPU
// (cuda/src/eri.cu:20-89): instead of an AoS of basis functions plus a
// CPU-side Schwarz table, the job keeps in HBM
//   * one record per shell pair with its primitive-pair geometry and the
//     dense Hermite->Cartesian E matrices (weights and exp(-mu AB^2) folded),
//   * a Boys-function table (FP64, Taylor grid),
//   * the BF-level Schwarz table, computed on the device from the diagonal
//     shell quartets (the reference's schwarz_bounds, integrals.hpp:732-752,
//     runs on the CPU even on its GPU path, eri.cu:32),
//   * the screened list of unique shell quartets (the reference screens per
//     basis-function quartet, integrals.hpp:771),
// so that every Fock build is: upload density -> one work-queue launch ->
// symmetrise -> download, with no ERI storage.
#include "hfx_engine.hpp"

#include <algorithm>
#include <memory>
#include <thread>
#include <exception>
#include <atomic>
#include <cstdio>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <tuple>
#include <map>
#include <mutex>
#include <numeric>

namespace hfx {

namespace {
constexpr size_t kPoolMaxBlock = size_t(256) << 20;
struct Pool {
    std::mutex mu;
    std::map<std::pair<int, size_t>, std::vector<void*>> free_blocks;   // (device, bucket) -> blocks
    size_t cached = 0;
};
Pool& pool()
{
    static Pool* p = new Pool();   // never destroyed: blocks live until the process exits
    return *p;
}
size_t bucket_of(size_t bytes)
{
    size_t b = 256;
    while (b < bytes) b <<= 1;
    return b;
}
}  // namespace

void* pool_alloc(size_t bytes)
{
    int dev = 0;
    cudaGetDevice(&dev);
    void* p = nullptr;
    if (bytes > kPoolMaxBlock) {
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            throw Error(HFX_ERR_OOM, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
        }
        return p;
    }
    const size_t b = bucket_of(bytes);
    {
        std::lock_guard<std::mutex> lk(pool().mu);
        auto it = pool().free_blocks.find({dev, b});
        if (it != pool().free_blocks.end() && !it->second.empty()) {
            p = it->second.back();
            it->second.pop_back();
            pool().cached -= b;
            return p;
        }
    }
    cudaError_t e = cudaMalloc(&p, b);
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw Error(HFX_ERR_OOM, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
    }
    return p;
}

void pool_free(void* p, size_t bytes)
{
    if (!p) return;
    if (bytes > kPoolMaxBlock) {
        cudaFree(p);
        return;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    const size_t b = bucket_of(bytes);
    std::lock_guard<std::mutex> lk(pool().mu);
    pool().free_blocks[{dev, b}].push_back(p);
    pool().cached += b;
}

size_t pool_cached_bytes()
{
    std::lock_guard<std::mutex> lk(pool().mu);
    return pool().cached;
}

void cuda_check(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) {
        cudaGetLastError();
        hfx_status code = (e == cudaErrorMemoryAllocation) ? HFX_ERR_OOM : HFX_ERR_CUDA;
        throw Error(code, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

static double flops_per_prim(int la, int lb, int lc, int ld)
{
    // algorithmic MD flop count per primitive quartet (boys + R + ket + bra + prefactor)
    int L1 = la + lb, L2 = lc + ld, L = L1 + L2;
    double boys = 12 + 3 * L;
    double R = 3.0 * (L + 1) * (L + 2) * (L + 3) * (L + 4) / 24.0;
    double ket = 2.0 * nherm(L1) * nherm(L2) * ncart(lc) * ncart(ld);
    double bra = 2.0 * nherm(L1) * ncart(la) * ncart(lb) * ncart(lc) * ncart(ld);
    return boys + R + ket + bra + 20;
}

Job::Job(Basis b, const hfx_options& opt) : basis_(std::move(b)), opt_(opt)
{
    frags_ = single_fragment(basis_);
    init(opt);
}

Job::Job(const std::vector<Basis>& mols, const hfx_options& opt) : opt_(opt)
{
    if (mols.empty() || mols.size() > 65535) throw Error(HFX_ERR_INVALID, "packed job: 1..65535 molecules");
    basis_ = concat_basis(mols, frags_);
    packed_ = true;
    init(opt);
}

void Job::set_active(const unsigned char* flags)
{
    if (!d_active_.p) throw Error(HFX_ERR_INVALID, "set_active: not a packed job");
    cuda_check(cudaMemcpyAsync(d_active_.p, flags, frags_.count(), cudaMemcpyHostToDevice, stream_), "active flags");
}

Basis concat_basis(const std::vector<Basis>& mols, Fragments& fr)
{
    Basis out;
    fr = Fragments{};
    fr.sh.push_back(0);
    fr.bf.push_back(0);
    fr.pbase.push_back(0);
    fr.moff.push_back(0);
    fr.qoff.push_back(0);
    for (const Basis& m : mols) {
        const int atom0 = (int)out.atom_Z.size();
        for (Shell sh : m.shells) {
            sh.bf0 += out.K;
            sh.atom += atom0;
            out.shells.push_back(std::move(sh));
        }
        out.K += m.K;
        out.atom_Z.insert(out.atom_Z.end(), m.atom_Z.begin(), m.atom_Z.end());
        out.atom_xyz.insert(out.atom_xyz.end(), m.atom_xyz.begin(), m.atom_xyz.end());
        const long long ns = (long long)m.shells.size();
        fr.sh.push_back((int)out.shells.size());
        fr.bf.push_back(out.K);
        fr.pbase.push_back(fr.pbase.back() + (int)(ns * (ns + 1) / 2));
        fr.moff.push_back(fr.moff.back() + (long long)m.K * m.K);
        fr.qoff.push_back(fr.qoff.back() + (long long)m.K * (m.K + 1) / 2);
    }
    return out;
}

Fragments single_fragment(const Basis& b)
{
    Fragments fr;
    const long long ns = (long long)b.shells.size();
    fr.sh = {0, (int)ns};
    fr.bf = {0, b.K};
    fr.pbase = {0, (int)(ns * (ns + 1) / 2)};
    fr.moff = {0, (long long)b.K * b.K};
    fr.qoff = {0, (long long)b.K * (b.K + 1) / 2};
    return fr;
}

void Job::init(const hfx_options& opt)
{
    opt_ = opt;
    if (opt_.screening_threshold == 0.0) opt_.screening_threshold = 1e-8;
    if (opt_.fp32_threshold == 0.0) opt_.fp32_threshold = 1e-7;
    device_ = opt_.device;
    no_graphs_ = std::getenv("HFX_NO_GRAPHS") != nullptr;
    int ndev = 0;
    cuda_check(cudaGetDeviceCount(&ndev), "cudaGetDeviceCount");
    if (device_ < 0 || device_ >= ndev) throw Error(HFX_ERR_INVALID, "invalid CUDA device ordinal");
    cuda_check(cudaSetDevice(device_), "cudaSetDevice");
    cuda_check(cudaDeviceGetAttribute(&nsm_, cudaDevAttrMultiProcessorCount, device_), "SM count");
    cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
    cuda_check(cudaEventCreate(&ev0_), "event");
    cuda_check(cudaEventCreate(&ev1_), "event");
    cuda_check(cudaEventCreate(&evk0_), "event");
    cuda_check(cudaEventCreate(&evk1_), "event");
    d_counter_.alloc(4);

    const std::vector<double>& tab = boys_table_host();
    d_boys_.upload(tab, stream_);
    d_boys32_.upload(boys_table32_host(), stream_);
    d_boys64_.upload(boys_table64_host(), stream_);
    for (int s = 0; s < 3; ++s) {
        cudaStream_t st;
        cuda_check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
        aux_.push_back(st);
        cudaEvent_t ev;
        cuda_check(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event");
        aux_ev_.push_back(ev);
    }
    cuda_check(cudaEventCreateWithFlags(&fork_ev_, cudaEventDisableTiming), "event");

    // HFX_TRACE_SETUP: phase times of job creation on stderr
    const bool trace = std::getenv("HFX_TRACE_SETUP") != nullptr;
    auto tnow = [] { return std::chrono::steady_clock::now(); };
    auto ms = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
        return std::chrono::duration<double, std::milli>(b - a).count();
    };
    auto t0 = tnow();
    build_pairs();
    auto t1 = tnow();
    compute_schwarz();
    auto t2 = tnow();
    {
        std::vector<float> q32(qbf_.begin(), qbf_.end());
        d_qbf32_.upload(q32, stream_);
    }
    // shell-pair Schwarz maxima into the device pair records (density screening)
    for (size_t p = 0; p < dpairs_host_.size(); ++p) dpairs_host_[p].qmax = qsh_[p];
    d_pairs_.upload(dpairs_host_, stream_);
    d_dsh_.alloc(std::max<size_t>(1, dpairs_host_.size()));
    {
        const int F = frags_.count();
        std::vector<int> fk(F);
        std::vector<long long> fm(F);
        for (int f = 0; f < F; ++f) {
            fk[f] = frags_.K(f);
            fm[f] = frags_.moff[f];
        }
        d_fk_.upload(fk, stream_);
        d_fmoff_.upload(fm, stream_);
        if (packed_) {
            std::vector<unsigned char> on(F, 1);
            d_active_.upload(on, stream_);
        }
    }
    auto t3 = tnow();
    build_jk_groups(false, gs_fp64_);
    auto t4 = tnow();
    if (mixed()) {
        build_jk_groups(true, gs_mixed_);
        // float density copies of the FP32 groups, allocated with the job so
        // that builds (the allocation-free entry point included) allocate nothing
        d_d32_.alloc((size_t)3 * nmat());
    }
    d_counters_.alloc(std::max<size_t>(1, std::max(gs_fp64_.groups.size(), gs_mixed_.groups.size())));
    cuda_check(cudaStreamSynchronize(stream_), "job setup");
    if (trace)
        std::fprintf(stderr, "job setup (K=%d): pairs %.1f ms, Schwarz %.1f ms, pair upload %.1f ms, FP64 plan %.1f ms, "
                             "rest %.1f ms\n",
                     basis_.K, ms(t0, t1), ms(t1, t2), ms(t2, t3), ms(t3, t4), ms(t4, tnow()));
}

Job::~Job()
{
    cudaSetDevice(device_);
    if (stream_) cudaStreamSynchronize(stream_);
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
    if (evk0_) cudaEventDestroy(evk0_);
    if (evk1_) cudaEventDestroy(evk1_);
    clear_graphs();
    for (auto e : aux_ev_) cudaEventDestroy(e);
    for (auto st : aux_) cudaStreamDestroy(st);
    if (fork_ev_) cudaEventDestroy(fork_ev_);
    if (stream_) cudaStreamDestroy(stream_);
}

const std::vector<double>& boys_table_host()
{
    // F_m(k/16) for m < kBoysM - 1 (converged series) and exp(-k/16) in the
    // last column; computed once per process (~70 ms of long-double series)
    static const std::vector<double> tab = [] {
        std::vector<double> t((size_t)kBoysN * kBoysM);
        for (int k = 0; k < kBoysN; ++k) {
            for (int m = 0; m < kBoysM - 1; ++m) t[(size_t)k * kBoysM + m] = boys_host(m, (double)k / kBoysInvStep);
            t[(size_t)k * kBoysM + kBoysM - 1] = std::exp(-(double)k / kBoysInvStep);
        }
        return t;
    }();
    return tab;
}

const std::vector<double>& boys_table64_host()
{
    static const std::vector<double> t64 = [] {
        const std::vector<double>& t = boys_table_host();
        std::vector<double> v((size_t)(kBoys64MaxL + 1) * kBoysN * kBoys64Row, 0.0);
        double fac = 1.0;
        double inv_fact[7];
        for (int j = 0; j < 7; ++j) {
            inv_fact[j] = 1.0 / fac;
            fac *= (double)(j + 1);
        }
        for (int L = 0; L <= kBoys64MaxL; ++L)
            for (int k = 0; k < kBoysN; ++k) {
                double* r = &v[((size_t)L * kBoysN + k) * kBoys64Row];
                for (int j = 0; j < 7; ++j) r[j] = t[(size_t)k * kBoysM + L + j] * inv_fact[j];
                r[7] = t[(size_t)k * kBoysM + (kBoysM - 1)];
            }
        return v;
    }();
    return t64;
}

const std::vector<float>& boys_table32_host()
{
    static const std::vector<float> t32 = [] {
        const std::vector<double>& t = boys_table_host();
        std::vector<float> v((size_t)(kBoys32MaxL + 1) * kBoysN * kBoys32Row, 0.0f);
        const double fac[5] = {1.0, 1.0, 0.5, 1.0 / 6.0, 1.0 / 24.0};
        for (int L = 0; L <= kBoys32MaxL; ++L)
            for (int k = 0; k < kBoysN; ++k) {
                float* r = &v[((size_t)L * kBoysN + k) * kBoys32Row];
                for (int j = 0; j < 5; ++j) r[j] = (float)(t[(size_t)k * kBoysM + L + j] * fac[j]);
                r[5] = (float)t[(size_t)k * kBoysM + (kBoysM - 1)];
            }
        return v;
    }();
    return t32;
}

// Task order of a launch group: largest cost first, so that the work queues
// hand out the long tasks early and the threads of a warp get tasks of about
// the same cost.  Counting sort on 1/16-octave cost bins (stable within a
// bin): O(n), where a comparison sort of a million-task plan took tens of
// milliseconds of job setup.
// With `shape` (thread-kernel groups: bra x ket primitive-pair counts of the
// task, 8 bits each), tasks of one cost bin are further ordered by shape, so
// that the 32 threads of a warp run loops of the same trip counts.
static std::vector<size_t> order_by_cost_desc(const std::vector<double>& cost,
                                              const std::vector<unsigned short>* shape = nullptr)
{
    constexpr int kBins = 1024;
    const size_t n = cost.size();
    std::vector<size_t> pre;   // stable pre-order by shape
    if (shape) {
        std::vector<size_t> cs(65537, 0);
        for (size_t i = 0; i < n; ++i) ++cs[(*shape)[i] + 1];
        for (int b = 0; b < 65536; ++b) cs[b + 1] += cs[b];
        pre.resize(n);
        for (size_t i = 0; i < n; ++i) pre[cs[(*shape)[i]]++] = i;
    }
    std::vector<unsigned short> bin(n);
    std::vector<size_t> count(kBins + 1, 0);
    for (size_t i = 0; i < n; ++i) {
        // 16 bins per octave: the exponent and the top four mantissa bits
        // (monotonic in the cost, which is all the order needs)
        const double c = cost[i] > 1.0 ? cost[i] : 1.0;
        unsigned long long bits;
        std::memcpy(&bits, &c, sizeof(bits));
        int b = (int)(((bits >> 52) - 1023) * 16 + ((bits >> 48) & 15));
        b = b < 0 ? 0 : (b >= kBins ? kBins - 1 : b);
        bin[i] = (unsigned short)(kBins - 1 - b);   // descending cost = ascending bin
        ++count[bin[i] + 1];
    }
    for (int b = 0; b < kBins; ++b) count[b + 1] += count[b];
    std::vector<size_t> idx(n);
    for (size_t r = 0; r < n; ++r) {
        const size_t i = shape ? pre[r] : r;
        idx[count[bin[i]]++] = i;
    }
    return idx;
}

// The classes whose class kernels split their ket component pairs over
// several threads per task (or, (dd|ss), hold 36 accumulators): in FP64 they
// beat the warp kernel on lightly contracted quartets (benzene/cc-pVDZ build
// 21.4 -> 17.9 ms) but not on heavily contracted ones (NaCl/cc-pVTZ 20.0 ->
// 22.2 ms), whose quartets the plan keeps on the warp kernel.
static bool is_ket_blocked_class(int pcb, int pck)
{
    static const int blocked[][2] = {{2, 2}, {3, 2}, {4, 1}, {4, 2}, {4, 3}, {4, 4}, {5, 0}, {5, 1}, {5, 2}, {5, 3}};
    for (auto& c : blocked)
        if (c[0] == pcb && c[1] == pck) return true;
    return false;
}

bool is_small_class(int pcb, int pck)
{
    // every class up to (dd|ds) with at most d functions, in both precisions;
    // the larger ones split their ket component pairs over several threads
    // per task
    static const int small[][2] = {{0, 0}, {1, 0}, {1, 1}, {2, 0}, {2, 1}, {3, 0}, {3, 1}, {3, 3}, {4, 0},
                                   {2, 2}, {3, 2}, {4, 1}, {4, 2}, {4, 3}, {4, 4}, {5, 0}, {5, 1}, {5, 2}, {5, 3}};
    for (auto& c : small)
        if (c[0] == pcb && c[1] == pck) return true;
    return false;
}

static int pair_class(int l0, int l1) { return l0 * (l0 + 1) / 2 + l1; }

const ClassTables& class_tables()
{
    static ClassTables ct = [] {
        ClassTables t;
        for (int l0 = 0; l0 <= kMaxL; ++l0)
            for (int l1 = 0; l1 <= l0; ++l1) {
                PairClassTab pt{};
                int n0 = ncart(l0), n1 = ncart(l1);
                pt.nab = n0 * n1;
                pt.ab_off = (int)t.ab_start.size();
                pt.k_off = (int)t.k_herm.size();
                int k = 0;
                for (int a = 0; a < n0; ++a)
                    for (int b = 0; b < n1; ++b) {
                        t.ab_start.push_back(k);
                        int ax, ay, az, bx, by, bz;
                        component(l0, a, ax, ay, az);
                        component(l1, b, bx, by, bz);
                        for (int tt = 0; tt <= ax + bx; ++tt)
                            for (int u = 0; u <= ay + by; ++u)
                                for (int v = 0; v <= az + bz; ++v, ++k) {
                                    t.k_herm.push_back((short)herm_index(tt, u, v));
                                    t.k_lin.push_back((short)((tt * 169 + u * 13 + v) | (((tt + u + v) & 1) << 14)));
                                }
                    }
                t.ab_start.push_back(k);
                pt.ncoef = k;
                pt.stride = (5 + k + 3) & ~3;   // rec_stride (hfx_class.cuh): 16-byte aligned records
                t.tab.push_back(pt);
            }
        return t;
    }();
    return ct;
}

// Primitive pairs below this fraction of their shell pair's largest
// coefficient are left out (build_pair_data).
constexpr double kPrimPairCut = 1e-18;

namespace {
// f(i) for i in [0, n) on up to 16 host threads, indices handed out one at a
// time; the first exception is rethrown after every thread has joined.
template <typename F>
void parallel_for(int n, F&& f)
{
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    const int nt = std::min(std::min(n, hw), 16);
    if (nt <= 1) {
        for (int i = 0; i < n; ++i) f(i);
        return;
    }
    std::atomic<int> next{0};
    std::exception_ptr err;
    std::mutex emu;
    auto work = [&] {
        for (;;) {
            const int i = next.fetch_add(1);
            if (i >= n) return;
            try {
                f(i);
            } catch (...) {
                std::lock_guard<std::mutex> lk(emu);
                if (!err) err = std::current_exception();
            }
        }
    };
    std::vector<std::thread> pool;
    pool.reserve(nt - 1);
    for (int t = 1; t < nt; ++t) pool.emplace_back(work);
    work();
    for (auto& th : pool) th.join();
    if (err) std::rethrow_exception(err);
}
}  // namespace

PairData build_pair_data(const Basis& basis, const Fragments& fr)
{
    const ClassTables& ct = class_tables();
    const auto& sh = basis.shells;
    // the shell pairs in their final order; each is built on its own (host
    // threads), then appended in that order, so the tables do not depend on
    // the thread count
    struct Item {
        int f, A, B;
    };
    std::vector<Item> items;
    for (int f = 0; f < fr.count(); ++f)
        for (int A = fr.sh[f]; A < fr.sh[f + 1]; ++A)
            for (int B = fr.sh[f]; B <= A; ++B) items.push_back(Item{f, A, B});
    struct PairOut {
        std::vector<PairGeo> geo;
        std::vector<double> epool, rec;
    };
    std::vector<PairOut> outs(items.size());
    constexpr int kPairsPerUnit = 16;
    parallel_for((int)((items.size() + kPairsPerUnit - 1) / kPairsPerUnit), [&](int u) {
        std::vector<double> Ex, Ey, Ez;
        const size_t i1 = std::min(items.size(), (size_t)(u + 1) * kPairsPerUnit);
        for (size_t it = (size_t)u * kPairsPerUnit; it < i1; ++it) {
            int s0 = items[it].A, s1 = items[it].B;
            if (sh[s0].L < sh[s1].L) std::swap(s0, s1);
            const Shell& S0 = sh[s0];
            const Shell& S1 = sh[s1];
            const int l0 = S0.L, l1 = S1.L, L = l0 + l1;
            const int n0 = ncart(l0), n1 = ncart(l1), H = nherm(L);
            const PairClassTab& pt = ct.tab[pair_class(l0, l1)];
            const int nt = L + 1;
            // All primitive pairs of the shell pair first (geometry, dense E
            // block, record coefficients), then only those whose largest
            // Hermite->Cartesian coefficient reaches kPrimPairCut of the shell
            // pair's largest: the others (tight primitives on distant centres,
            // exp(-mu |AB|^2) ~ 0) change no integral by more than ~1e-14 of
            // its size, and skipping them removes their primitive quartets
            // from every class kernel.
            const int np = S0.nprim() * S1.nprim();
            const size_t ne = (size_t)n0 * n1 * H;
            std::vector<double> pgeo((size_t)np * 4), pe((size_t)np * ne, 0.0), pc((size_t)np * pt.ncoef), pmax(np, 0.0);
            std::vector<int> pnc(np, 0);
            double cmax_pair = 0.0;
            for (int i = 0; i < S0.nprim(); ++i)
                for (int j = 0; j < S1.nprim(); ++j) {
                    const int q = i * S1.nprim() + j;
                    const double a = S0.exps[i], be = S1.exps[j], p = a + be;
                    hermite_1d(l0, l1, a, be, S0.x, S1.x, Ex);
                    hermite_1d(l0, l1, a, be, S0.y, S1.y, Ey);
                    hermite_1d(l0, l1, a, be, S0.z, S1.z, Ez);
                    pgeo[4 * q] = p;
                    pgeo[4 * q + 1] = (a * S0.x + be * S1.x) / p;
                    pgeo[4 * q + 2] = (a * S0.y + be * S1.y) / p;
                    pgeo[4 * q + 3] = (a * S0.z + be * S1.z) / p;
                    double cmax = 0.0;
                    int nc = 0;
                    double* cq = pc.data() + (size_t)q * pt.ncoef;
                    for (int c0 = 0; c0 < n0; ++c0) {
                        int ax, ay, az;
                        component(l0, c0, ax, ay, az);
                        for (int c1 = 0; c1 < n1; ++c1) {
                            int bx, by, bz;
                            component(l1, c1, bx, by, bz);
                            const double w = S0.w[(size_t)c0 * S0.nprim() + i] * S1.w[(size_t)c1 * S1.nprim() + j];
                            double* row = pe.data() + (size_t)q * ne + (size_t)(c0 * n1 + c1) * H;
                            for (int t = 0; t <= ax + bx; ++t)
                                for (int u2 = 0; u2 <= ay + by; ++u2)
                                    for (int v = 0; v <= az + bz; ++v) {
                                        const double c = w * Ex[((size_t)ax * (l1 + 1) + bx) * nt + t] *
                                                         Ey[((size_t)ay * (l1 + 1) + by) * nt + u2] *
                                                         Ez[((size_t)az * (l1 + 1) + bz) * nt + v];
                                        row[herm_index(t, u2, v)] = c;
                                        cq[nc++] = c;
                                        cmax = std::max(cmax, std::fabs(c));
                                    }
                        }
                    }
                    pnc[q] = nc;
                    pmax[q] = cmax;
                    cmax_pair = std::max(cmax_pair, cmax);
                }
            PairOut& o = outs[it];
            for (int q = 0; q < np; ++q) {
                if (pmax[q] < kPrimPairCut * cmax_pair) continue;
                o.geo.push_back(make_pairgeo(pgeo[4 * q], pgeo[4 * q + 1], pgeo[4 * q + 2], pgeo[4 * q + 3]));
                o.epool.insert(o.epool.end(), pe.begin() + (size_t)q * ne, pe.begin() + (size_t)(q + 1) * ne);
                const size_t rb = o.rec.size();
                o.rec.resize(rb + pt.stride, 0.0);
                o.rec[rb] = pgeo[4 * q];
                o.rec[rb + 1] = pgeo[4 * q + 1];
                o.rec[rb + 2] = pgeo[4 * q + 2];
                o.rec[rb + 3] = pgeo[4 * q + 3];
                o.rec[rb + 4] = 1.0 / pgeo[4 * q];
                for (int k = 0; k < pnc[q]; ++k) o.rec[rb + 5 + k] = pc[(size_t)q * pt.ncoef + k];
            }
        }
    });
    PairData pd;
    {
        size_t ng = 0, nep = 0, nrec = 0;
        for (const PairOut& o : outs) {
            ng += o.geo.size();
            nep += o.epool.size();
            nrec += o.rec.size();
        }
        pd.geo.reserve(ng);
        pd.epool.reserve(nep);
        pd.rec.reserve(nrec);
    }
    for (size_t it = 0; it < items.size(); ++it) {
        const int f = items[it].f, A = items[it].A, B = items[it].B;
        int s0 = A, s1 = B;
        if (sh[A].L < sh[B].L) std::swap(s0, s1);
        const Shell& S0 = sh[s0];
        const Shell& S1 = sh[s1];
        const int l0 = S0.L, l1 = S1.L;
        PairOut& o = outs[it];
        HostPair hp{};
        hp.frag = f;
        hp.s0 = s0;
        hp.s1 = s1;
        hp.l0 = l0;
        hp.l1 = l1;
        hp.same = (A == B);
        hp.pp0 = (int)pd.geo.size();
        hp.e_off = (long long)pd.epool.size();
        hp.npp = (int)o.geo.size();
        const long long rec_off = (long long)pd.rec.size();
        pd.geo.insert(pd.geo.end(), o.geo.begin(), o.geo.end());
        pd.epool.insert(pd.epool.end(), o.epool.begin(), o.epool.end());
        pd.rec.insert(pd.rec.end(), o.rec.begin(), o.rec.end());
        PairOut().geo.swap(o.geo);
        std::vector<double>().swap(o.epool);
        std::vector<double>().swap(o.rec);
        DPair d{};
        d.bf0 = S0.bf0 - fr.bf[f];
        d.bf1 = S1.bf0 - fr.bf[f];
        d.l0 = l0;
        d.l1 = l1;
        d.pp0 = hp.pp0;
        d.npp = hp.npp;
        d.e_off = hp.e_off;
        d.same = hp.same ? 1 : 0;
        d.id = (int)pd.hpairs.size();
        d.qmax = 0.0;
        d.rec_off = rec_off;
        d.pc = pair_class(l0, l1);
        d.sh0 = s0 - fr.sh[f];
        d.sh1 = s1 - fr.sh[f];
        d.kdim = fr.K(f);
        d.pbase = fr.pbase[f];
        d.frag = f;
        d.moff = fr.moff[f];
        d.qoff = fr.qoff[f];
        pd.dpairs.push_back(d);
        pd.hpairs.push_back(hp);
    }
    return pd;
}

void Job::build_pairs()
{
    PairData pd = build_pair_data(basis_, frags_);
    hpairs_ = std::move(pd.hpairs);
    dpairs_host_ = pd.dpairs;
    d_pairs_.upload(pd.dpairs, stream_);
    d_ppgeo_.upload(pd.geo, stream_);
    d_epool_.upload(pd.epool, stream_);
    d_rec64_.upload(pd.rec, stream_);
    std::vector<float> r32(pd.rec.begin(), pd.rec.end());
    d_rec32_.upload(r32, stream_);
    const ClassTables& ct = class_tables();
    d_pct_.upload(ct.tab, stream_);
    d_abs_.upload(ct.ab_start, stream_);
    d_kh_.upload(ct.k_herm, stream_);
    d_kl_.upload(ct.k_lin, stream_);
    cuda_check(cudaStreamSynchronize(stream_), "pair upload");
}

LaunchArgs Job::base_args() const
{
    LaunchArgs a{};
    a.pairs = d_pairs_.p;
    a.pp_geo = d_ppgeo_.p;
    a.epool = d_epool_.p;
    a.boys = d_boys_.p;
    a.counter = d_counter_.p;
    a.K = basis_.K;
    a.thr = opt_.screening_threshold;
    a.Qbf = d_qbf_.p;
    return a;
}

void Job::run_eri_tasks(const DevBuf<Task>& tasks, int ntasks, int maxacc, int maxw, int maxr, LaunchArgs a)
{
    if (ntasks == 0) return;
    a.tasks = tasks.p;
    a.ntasks = ntasks;
    cuda_check(cudaMemsetAsync(d_counter_.p, 0, sizeof(int), stream_), "memset counter");
    size_t sm = generic_smem_bytes(maxacc, maxw, maxr);
    int per_sm = (int)std::max<size_t>(1, std::min<size_t>(16, (220 * 1024) / std::max<size_t>(sm, 1)));
    int grid = std::min(ntasks, nsm_ * per_sm);
    cuda_check(launch_eri(a, maxacc, maxw, maxr, grid, stream_), "ERI kernel launch");
}

void Job::compute_schwarz()
{
    // Diagonal shell quartets (AB|AB) on the warp kernel (NK = 0 writes the
    // BF-pair bounds sqrt((ab|ab)) and the per-pair maximum), tiered by the
    // shared-memory slice each class needs.
    const int np = (int)hpairs_.size();
    size_t npair_bf = (size_t)frags_.qoff.back();
    d_qbf_.alloc(npair_bf);
    d_qsh_.alloc(np);
    cuda_check(cudaMemsetAsync(d_qbf_.p, 0, npair_bf * sizeof(double), stream_), "memset");
    cuda_check(cudaMemsetAsync(d_qsh_.p, 0, np * sizeof(unsigned long long), stream_), "memset");
    std::map<int, std::vector<Task>> tiers;
    std::map<int, int> tier_slice;
    for (int p = 0; p < np; ++p) {
        const HostPair& h = hpairs_[p];
        int sl = warp_slice_elems(h.l0, h.l1, h.l0, h.l1, h.npp, kDefaultLaneMinNpp);
        int tier = 0;
        while ((512 << tier) < sl) ++tier;
        tiers[tier].push_back(make_task(p, p, 0, h.npp, 0, h.npp));   // whole quartet: the pass writes, not adds
        tier_slice[tier] = std::max(tier_slice[tier], sl);
    }
    std::vector<DevBuf<Task>> dts(tiers.size());
    DevBuf<int> ctr;
    ctr.alloc(tiers.size());
    cuda_check(cudaMemsetAsync(ctr.p, 0, sizeof(int) * tiers.size(), stream_), "memset");
    size_t ti = 0;
    for (auto& kv : tiers) {
        dts[ti].upload(kv.second, stream_);
        const int slice = (tier_slice[kv.first] + 1) & ~1;
        const int wpc = (int)std::max<size_t>(1, std::min<size_t>(8, (200 * 1024 - kWarpSmemHeader) / (slice * sizeof(double))));
        const size_t sm = kWarpSmemHeader + sizeof(double) * (size_t)slice * wpc;
        const int ctas_per_sm = (int)std::max<size_t>(1, (228 * 1024) / (sm + 1024));
        const long long need = ((long long)kv.second.size() + wpc - 1) / wpc;
        const int grid = (int)std::min<long long>(need, (long long)nsm_ * ctas_per_sm);
        WarpArgs<double> a{};
        a.pairs = d_pairs_.p;
        a.rec = d_rec64_.p;
        a.pct = d_pct_.p;
        a.ab_start = d_abs_.p;
        a.k_herm = d_kh_.p;
        a.k_lin = d_kl_.p;
        a.tasks = dts[ti].p;
        a.ntasks = (int)kv.second.size();
        a.counter = ctr.p + ti;
        a.boys = d_boys64_.p;
        a.thr = -1.0;
        a.K = basis_.K;
        a.slice = slice;
        a.lane_min_npp = kDefaultLaneMinNpp;
        a.Qout_bf = d_qbf_.p;
        a.Qout_sh = d_qsh_.p;
        cuda_check(launch_warp(false, &a, 0, grid, wpc, stream_), "schwarz launch");
        ++ti;
    }
    qbf_.resize(npair_bf);
    std::vector<unsigned long long> qs(np);
    cuda_check(cudaMemcpyAsync(qbf_.data(), d_qbf_.p, npair_bf * sizeof(double), cudaMemcpyDeviceToHost, stream_),
               "download Q");
    cuda_check(cudaMemcpyAsync(qs.data(), d_qsh_.p, np * sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream_),
               "download Q");
    cuda_check(cudaStreamSynchronize(stream_), "schwarz");
    qsh_.resize(np);
    for (int p = 0; p < np; ++p) {
        double v;
        std::memcpy(&v, &qs[p], sizeof(double));
        qsh_[p] = v;
    }
}

void Job::schwarz_host(std::vector<double>& Q) const { Q = qbf_; }

// Calls f(X, Y) for every unique shell-pair pair X >= Y of the same molecule
// with Q_X Q_Y >= thr (all pairs if thr < 0), visiting only the survivors:
// a molecule's pairs are scanned in decreasing Q order and the scan for X
// stops at the first Q_Y below thr / Q_X.
template <typename F>
void Job::for_each_surviving_quartet(double thr, F&& f) const
{
    for (int fr = 0; fr < frags_.count(); ++fr) {
        const int p0 = frags_.pbase[fr], p1 = frags_.pbase[fr + 1];
        if (thr < 0.0) {
            for (int X = p0; X < p1; ++X)
                for (int Y = p0; Y <= X; ++Y) f(X, Y);
            continue;
        }
        std::vector<int> order(p1 - p0);
        std::iota(order.begin(), order.end(), p0);
        std::sort(order.begin(), order.end(), [&](int a, int b) { return qsh_[a] > qsh_[b]; });
        for (int X = p0; X < p1; ++X) {
            if (qsh_[X] <= 0.0) continue;
            const double need = thr / qsh_[X];
            for (int Y : order) {
                if (qsh_[Y] < need) break;
                if (Y <= X) f(X, Y);
            }
        }
    }
}

void Job::build_tasks(double thr, std::vector<Task>& tasks, int& maxacc, int& maxw, int& maxr, double* flops,
                      double* prims) const
{
    // order pairs so that the pair with the larger (L, l0) is the bra
    auto key = [&](int p) { return (hpairs_[p].l0 + hpairs_[p].l1) * 16 + hpairs_[p].l0; };
    std::vector<double> cost;
    tasks.clear();
    maxacc = maxw = maxr = 1;
    for_each_surviving_quartet(thr, [&](int X, int Y) {
        int bra = X, ket = Y;
        if (key(Y) > key(X)) std::swap(bra, ket);
        tasks.push_back(make_task(bra, ket, 0, hpairs_[bra].npp, 0, hpairs_[ket].npp));
    });
    std::vector<double> c(tasks.size());
    double fsum = 0.0, psum = 0.0;
    for (size_t t = 0; t < tasks.size(); ++t) {
        const HostPair& b = hpairs_[tasks[t].bra];
        const HostPair& k = hpairs_[tasks[t].ket];
        c[t] = (double)b.npp * k.npp * flops_per_prim(b.l0, b.l1, k.l0, k.l1);
        fsum += c[t];
        psum += (double)b.npp * k.npp;
        int L1 = b.l0 + b.l1, L2 = k.l0 + k.l1;
        int nab = ncart(b.l0) * ncart(b.l1), ncd = ncart(k.l0) * ncart(k.l1);
        maxacc = std::max(maxacc, nab * ncd);
        maxw = std::max(maxw, nherm(L1) * ncd);
        maxr = std::max(maxr, nherm(L1 + L2));
    }
    if (flops) *flops = fsum;
    if (prims) *prims = psum;
    std::vector<size_t> idx(tasks.size());
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](size_t x, size_t y) { return c[x] > c[y]; });
    std::vector<Task> sorted(tasks.size());
    for (size_t t = 0; t < idx.size(); ++t) sorted[t] = tasks[idx[t]];
    tasks.swap(sorted);
}


// FP64 quartets of the ket-blocked classes with more primitive quartets than
// this run on the warp kernel.
constexpr long long kKetBlockMaxPrims64 = 64;

void Job::build_jk_groups(bool mixed, GroupSet& gs)
{
    clear_graphs();   // graphs hold the previous plan's task pointers
    const double thr = opt_.screening_threshold;
    const double tau = opt_.fp32_threshold;
    const int np = (int)hpairs_.size();
    // per shell pair: its class; per class pair: kernel form and algorithmic
    // flops per primitive quartet
    std::vector<unsigned char> pcls(np);
    for (int p = 0; p < np; ++p) pcls[p] = (unsigned char)pair_class(hpairs_[p].l0, hpairs_[p].l1);
    constexpr int kPC = (kMaxL + 1) * (kMaxL + 2) / 2;
    int pl0[kPC], pl1[kPC];
    for (int l0 = 0; l0 <= kMaxL; ++l0)
        for (int l1 = 0; l1 <= l0; ++l1) {
            pl0[pair_class(l0, l1)] = l0;
            pl1[pair_class(l0, l1)] = l1;
        }
    bool small_ok[kPC][kPC];
    bool ket_blocked[kPC][kPC];   // the ten classes beyond the nine single-block ones
    double fpp_tab[kPC][kPC];
    for (int a = 0; a < kPC; ++a)
        for (int b = 0; b < kPC; ++b) {
            small_ok[a][b] = is_small_class(a, b);
            ket_blocked[a][b] = is_ket_blocked_class(a, b);
            fpp_tab[a][b] = flops_per_prim(pl0[a], pl1[a], pl0[b], pl1[b]);
        }
    // buckets: small classes per (fp32, pcb, pck) at fp32 * 100 + pcb * 10 + pck;
    // the warp kernel's per fp32 at kWarpBucket + fp32
    constexpr int kWarpBucket = 200, kBuckets = 202;
    // Work units of the enumeration: ranges of bra-side shell pairs X of one
    // molecule.  Every unit lists its surviving quartets per bucket in the
    // serial visiting order (X ascending, Y by decreasing Schwarz bound), so
    // that the units concatenated in order give the same lists, and the same
    // plan, on any number of threads.
    struct Unit {
        int frag = 0, x0 = 0, x1 = 0;
        std::vector<std::vector<std::pair<int, int>>> q;   // per bucket: (bra, ket)
        std::vector<double> prims;                         // per bucket: primitive quartets
        std::vector<std::vector<Task>> t;                  // per bucket: tiles
        std::vector<std::vector<double>> cost;
        std::vector<std::vector<unsigned short>> shape;   // (bra, ket) primitive pairs of a task, 8 bits each
    };
    constexpr int kUnitPairs = 24;
    std::vector<Unit> units;
    std::vector<std::vector<int>> qorder(frags_.count());
    for (int fr = 0; fr < frags_.count(); ++fr) {
        const int p0 = frags_.pbase[fr], p1 = frags_.pbase[fr + 1];
        std::vector<int>& order = qorder[fr];
        order.resize(p1 - p0);
        std::iota(order.begin(), order.end(), p0);
        std::sort(order.begin(), order.end(), [&](int a, int b) { return qsh_[a] > qsh_[b]; });
        for (int x = p0; x < p1; x += kUnitPairs) {
            units.emplace_back();
            units.back().frag = fr;
            units.back().x0 = x;
            units.back().x1 = std::min(p1, x + kUnitPairs);
        }
    }
    const int nu = (int)units.size();
    const auto tp0 = std::chrono::steady_clock::now();
    parallel_for(nu, [&](int u) {
        Unit& un = units[u];
        un.q.resize(kBuckets);
        un.prims.assign(kBuckets, 0.0);
        const std::vector<int>& order = qorder[un.frag];
        for (int X = un.x0; X < un.x1; ++X) {
            if (qsh_[X] <= 0.0) continue;
            const double need = thr / qsh_[X];
            for (int Y : order) {
                if (qsh_[Y] < need) break;
                if (Y > X) continue;
                const double bound = qsh_[X] * qsh_[Y];
                int bra = X, ket = Y;
                if (pcls[Y] > pcls[X]) std::swap(bra, ket);
                const int f32 = mixed && bound < tau ? 1 : 0;
                const int pcb = pcls[bra], pck = pcls[ket];
                // FP64 quartets of the ket-block classes with many primitive
                // quartets go to the warp kernel: every ket block of a class
                // kernel task recomputes R and the Boys function
                const bool sm = small_ok[pcb][pck] &&
                                (f32 || !ket_blocked[pcb][pck] ||
                                 (long long)hpairs_[bra].npp * hpairs_[ket].npp <= kKetBlockMaxPrims64);
                const int b = sm ? f32 * 100 + pcb * 10 + pck : kWarpBucket + f32;
                un.q[b].push_back({bra, ket});
                un.prims[b] += (double)hpairs_[bra].npp * hpairs_[ket].npp;
            }
        }
    });
    std::vector<double> bprims(kBuckets, 0.0);
    for (const Unit& un : units)
        for (int b = 0; b < kBuckets; ++b) bprims[b] += un.prims[b];
    // Tiles of primitive quartets.  A thread task holds at most
    // shape_.small_chunk primitive quartets and a warp task at most
    // shape_.warp_chunk; a launch group with too few primitive quartets to
    // give every SM several CTAs' worth of tasks at that size is cut finer
    // (down to kMinThreadTile / kMinWarpTile), because a quartet list of a
    // few thousand long tasks leaves most SMs idle.  Thread tasks split the
    // bra primitive pairs first, then the ket ones; warp tasks split the bra
    // primitive pairs only, so that each warp task keeps its whole ket
    // contraction (the bra transform is applied once per bra primitive pair
    // over the ket sum).
    constexpr double kThreadFill = 4.0 * 128;   // threads per SM the thread-kernel groups should offer
    constexpr double kWarpFill = 16.0;          // warps per SM for the warp-kernel groups
    constexpr long long kMinThreadTile = 8, kMinWarpTile = 64;
    std::vector<long long> chunk(kBuckets, 1);
    for (int b = 0; b < kBuckets; ++b) {
        const bool sm = b < kWarpBucket;
        const double fill = (sm ? kThreadFill : kWarpFill) * nsm_;
        const long long cap = sm ? shape_.small_chunk : shape_.warp_chunk;
        const long long lo = sm ? kMinThreadTile : kMinWarpTile;
        chunk[b] = std::max<long long>(std::min<long long>(lo, cap),
                                       std::min<long long>(cap, (long long)std::ceil(bprims[b] / fill)));
    }
    const auto tp1 = std::chrono::steady_clock::now();
    parallel_for(nu, [&](int u) {
        Unit& un = units[u];
        un.t.resize(kBuckets);
        un.cost.resize(kBuckets);
        un.shape.resize(kBuckets);
        for (int bkt = 0; bkt < kBuckets; ++bkt) {
            const bool sm = bkt < kWarpBucket;
            const long long c = chunk[bkt];
            for (const auto& bq : un.q[bkt]) {
                const HostPair& b = hpairs_[bq.first];
                const HostPair& k = hpairs_[bq.second];
                const double fpp = fpp_tab[pcls[bq.first]][pcls[bq.second]];
                const long long pq = (long long)b.npp * k.npp;
                const long long n = std::max<long long>(1, (pq + c - 1) / c);
                const int nb = (int)std::min<long long>(b.npp, n);
                const int nk = sm ? (int)std::min<long long>(k.npp, (n + nb - 1) / nb) : 1;
                for (int x = 0; x < nb; ++x) {
                    const int i0 = (int)((long long)b.npp * x / nb), i1 = (int)((long long)b.npp * (x + 1) / nb);
                    for (int y = 0; y < nk; ++y) {
                        const int k0 = (int)((long long)k.npp * y / nk), k1 = (int)((long long)k.npp * (y + 1) / nk);
                        un.t[bkt].push_back(make_task(bq.first, bq.second, i0, i1, k0, k1));
                        un.cost[bkt].push_back((double)(i1 - i0) * (k1 - k0) * fpp);
                        if (sm)
                            un.shape[bkt].push_back(
                                (unsigned short)(std::min(i1 - i0, 255) * 256 + std::min(k1 - k0, 255)));
                    }
                }
            }
            std::vector<std::pair<int, int>>().swap(un.q[bkt]);
        }
    });
    // per bucket: the units' tiles in unit order, then ordered by cost
    struct Bucket {
        std::vector<Task> t;
        std::vector<double> cost;
        std::vector<unsigned short> shape;
        std::vector<size_t> order;
    };
    std::vector<Bucket> bk(kBuckets);
    const auto tp2 = std::chrono::steady_clock::now();
    parallel_for(kBuckets, [&](int b) {
        size_t n = 0;
        for (const Unit& un : units) n += un.t[b].size();
        if (n == 0) return;
        Bucket& B = bk[b];
        B.t.reserve(n);
        B.cost.reserve(n);
        if (b < kWarpBucket) B.shape.reserve(n);
        for (Unit& un : units) {
            B.t.insert(B.t.end(), un.t[b].begin(), un.t[b].end());
            B.cost.insert(B.cost.end(), un.cost[b].begin(), un.cost[b].end());
            B.shape.insert(B.shape.end(), un.shape[b].begin(), un.shape[b].end());
            std::vector<Task>().swap(un.t[b]);
            std::vector<double>().swap(un.cost[b]);
            std::vector<unsigned short>().swap(un.shape[b]);
        }
        B.order = order_by_cost_desc(B.cost, B.shape.empty() ? nullptr : &B.shape);
    });
    const auto tp3 = std::chrono::steady_clock::now();
    // Launch groups: one per small-class bucket, then the warp buckets split
    // into tiers by the per-warp shared-memory slice their tasks need (powers
    // of two, so that tasks with small slices are not held to the occupancy
    // of the largest one).  Each group is a list of (bucket, index) in cost
    // order; their tasks are copied into the final array by parallel chunks.
    struct Span {
        int bucket;
        std::vector<size_t> idx;   // empty: the bucket's whole cost order
    };
    std::vector<LaunchGroup>& groups = gs.groups;
    groups.clear();
    std::vector<Span> spans;
    for (int f = 0; f < 2; ++f)
        for (int pcb = 0; pcb < 10; ++pcb)
            for (int pck = 0; pck <= pcb; ++pck) {
                const int b = f * 100 + pcb * 10 + pck;
                if (bk[b].t.empty()) continue;
                LaunchGroup g{};
                g.kind = 0;
                g.pcb = pcb;
                g.pck = pck;
                g.fp32 = f == 1;
                g.n = bk[b].t.size();
                groups.push_back(g);
                spans.push_back(Span{b, {}});
            }
    const size_t elem[2] = {sizeof(double), sizeof(float)};
    for (int f = 0; f < 2; ++f) {
        const Bucket& B = bk[kWarpBucket + f];
        if (B.t.empty()) continue;
        const size_t n = B.t.size();
        std::vector<int> sl(n);
        parallel_for((int)((n + 65535) / 65536), [&](int c) {
            for (size_t i = (size_t)c * 65536; i < std::min(n, (size_t)(c + 1) * 65536); ++i) {
                const HostPair& hb = hpairs_[B.t[i].bra];
                const HostPair& hk = hpairs_[B.t[i].ket];
                sl[i] = warp_slice_elems(hb.l0, hb.l1, hk.l0, hk.l1, B.t[i].k1 - B.t[i].k0, shape_.lane_min_npp);
            }
        });
        std::map<int, std::pair<std::vector<size_t>, int>> tiers;   // tier -> (indices in cost order, max slice)
        for (size_t i : B.order) {
            int tier = 0;
            while ((512 << tier) < sl[i]) ++tier;
            auto& tr = tiers[tier];
            tr.first.push_back(i);
            tr.second = std::max(tr.second, sl[i]);
        }
        for (auto& kv : tiers) {
            LaunchGroup g{};
            g.kind = 1;
            g.fp32 = f == 1;
            g.n = kv.second.first.size();
            g.slice = (kv.second.second + 1) & ~1;
            g.lane_min_npp = shape_.lane_min_npp;
            g.warps_per_cta = (int)std::max<size_t>(
                1, std::min<size_t>((size_t)shape_.warp_max_warps, (200 * 1024 - kWarpSmemHeader) / (g.slice * elem[f])));
            size_t sm = kWarpSmemHeader + elem[f] * (size_t)g.slice * g.warps_per_cta;
            int ctas_per_sm = (int)std::max<size_t>(1, (228 * 1024) / (sm + 1024));
            long long need = ((long long)g.n + g.warps_per_cta - 1) / g.warps_per_cta;
            g.grid = (int)std::min<long long>(need, (long long)nsm_ * ctas_per_sm);
            groups.push_back(g);
            spans.push_back(Span{kWarpBucket + f, std::move(kv.second.first)});
        }
    }
    size_t total = 0;
    for (LaunchGroup& g : groups) {
        g.off = total;
        total += g.n;
    }
    // copy in chunks of up to 65536 tasks; per chunk the flops, primitive
    // quartets and whole-quartet tiles, summed per group in chunk order
    struct Chunk {
        int group;
        size_t r0, r1;   // range within the group
        double flops = 0.0, prims = 0.0;
        long long whole = 0;
    };
    std::vector<Chunk> chunks;
    for (int gi = 0; gi < (int)groups.size(); ++gi)
        for (size_t r = 0; r < groups[gi].n; r += 65536)
            chunks.push_back(Chunk{gi, r, std::min(groups[gi].n, r + 65536)});
    std::unique_ptr<Task[]> all(new Task[std::max<size_t>(1, total)]);
    parallel_for((int)chunks.size(), [&](int c) {
        Chunk& ch = chunks[c];
        const Span& sp = spans[ch.group];
        const Bucket& B = bk[sp.bucket];
        Task* out = all.get() + groups[ch.group].off;
        for (size_t r = ch.r0; r < ch.r1; ++r) {
            const size_t i = sp.idx.empty() ? B.order[r] : sp.idx[r];
            const Task& t = B.t[i];
            out[r] = t;
            ch.flops += B.cost[i];
            ch.prims += (double)(t.i1 - t.i0) * (t.k1 - t.k0);
            if (t.i0 == 0 && t.k0 == 0) ++ch.whole;
        }
    });
    gs.flops64 = gs.flops32 = gs.prims = gs.quartets32 = 0.0;
    gs.nquartets = 0;
    for (const Chunk& ch : chunks) {
        LaunchGroup& g = groups[ch.group];
        g.flops += ch.flops;
        g.prims += ch.prims;
        gs.nquartets += (int)ch.whole;
        if (g.fp32) gs.quartets32 += (double)ch.whole;
    }
    for (const auto& g : groups) {
        if (g.fp32)
            gs.flops32 += g.flops;
        else
            gs.flops64 += g.flops;
        gs.prims += g.prims;
    }
    gs.ntasks = (int)total;
    const auto tp4 = std::chrono::steady_clock::now();
    gs.tasks.alloc(total);
    if (total > 0)
        cuda_check(cudaMemcpyAsync(gs.tasks.p, all.get(), total * sizeof(Task), cudaMemcpyHostToDevice, stream_),
                   "plan upload");
    // the host array is freed on return: the copy must have read it
    cuda_check(cudaStreamSynchronize(stream_), "plan upload");
    if (std::getenv("HFX_TRACE_SETUP")) {
        auto ms = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
            return std::chrono::duration<double, std::milli>(b - a).count();
        };
        const auto tp5 = std::chrono::steady_clock::now();
        std::fprintf(stderr, "plan (%s, %d tasks): enumerate %.1f ms, tile %.1f ms, order %.1f ms, assemble %.1f ms, "
                             "upload %.1f ms\n", mixed ? "mixed" : "fp64", gs.ntasks, ms(tp0, tp1), ms(tp1, tp2),
                     ms(tp2, tp3), ms(tp3, tp4), ms(tp4, tp5));
    }
}

StreamSink::StreamSink(cudaStream_t main, const std::vector<cudaStream_t>& aux, cudaEvent_t fork_ev,
                       const std::vector<cudaEvent_t>& aux_ev)
    : main_(main), aux_(aux), fork_ev_(fork_ev), aux_ev_(aux_ev)
{
}

void StreamSink::zero(int lane, void* p, size_t bytes)
{
    cuda_check(cudaMemsetAsync(p, 0, bytes, stream(lane)), "memset");
}

void StreamSink::kernel(int lane, const KernelSpec& s, void** params)
{
    if (s.grid.x == 0) return;
    cuda_check(cudaLaunchKernel(s.func, s.grid, s.block, params, s.smem, stream(lane)), "kernel launch");
}

void StreamSink::fork()
{
    cuda_check(cudaEventRecord(fork_ev_, main_), "fork");
    for (auto st : aux_) cuda_check(cudaStreamWaitEvent(st, fork_ev_, 0), "fork wait");
}

void StreamSink::join()
{
    for (size_t i = 0; i < aux_.size(); ++i) {
        cuda_check(cudaEventRecord(aux_ev_[i], aux_[i]), "join");
        cuda_check(cudaStreamWaitEvent(main_, aux_ev_[i], 0), "join wait");
    }
}

GraphSink::GraphSink(int lanes) : deps_(lanes) { cuda_check(cudaGraphCreate(&graph_, 0), "graph create"); }

GraphSink::~GraphSink()
{
    if (graph_) cudaGraphDestroy(graph_);
}

void GraphSink::zero(int lane, void* p, size_t bytes)
{
    cudaMemsetParams mp{};
    mp.dst = p;
    mp.value = 0;
    mp.elementSize = bytes % 4 == 0 ? 4 : 1;
    mp.width = bytes / mp.elementSize;
    mp.height = 1;
    mp.pitch = 0;
    cudaGraphNode_t node;
    std::vector<cudaGraphNode_t>& d = deps_[lane];
    cuda_check(cudaGraphAddMemsetNode(&node, graph_, d.data(), d.size(), &mp), "graph memset node");
    d.assign(1, node);
}

void GraphSink::kernel(int lane, const KernelSpec& s, void** params)
{
    if (s.grid.x == 0) return;
    cudaKernelNodeParams kp{};
    kp.func = const_cast<void*>(s.func);
    kp.gridDim = s.grid;
    kp.blockDim = s.block;
    kp.sharedMemBytes = (unsigned)s.smem;
    kp.kernelParams = params;
    kp.extra = nullptr;
    cudaGraphNode_t node;
    std::vector<cudaGraphNode_t>& d = deps_[lane];
    cuda_check(cudaGraphAddKernelNode(&node, graph_, d.data(), d.size(), &kp), "graph kernel node");
    d.assign(1, node);
}

void GraphSink::fork()
{
    for (size_t i = 1; i < deps_.size(); ++i) deps_[i] = deps_[0];
}

void GraphSink::join()
{
    std::vector<cudaGraphNode_t> all;
    for (const auto& d : deps_)
        for (auto n : d)
            if (std::find(all.begin(), all.end(), n) == all.end()) all.push_back(n);
    for (auto& d : deps_) d = all;
}

cudaGraphExec_t GraphSink::instantiate()
{
    cudaGraphExec_t exec = nullptr;
    cuda_check(cudaGraphInstantiate(&exec, graph_, 0), "graph instantiate");
    return exec;
}

void Job::launch_jk(OpSink& sk, int nk, const double* Dj, const double* Dk, const double* Dk2, double* J, double* Kx,
                    double* Kx2, int* counters, bool mixed_plan, double dthr)
{
    const GroupSet& gs = plan(mixed_plan);
    const std::vector<LaunchGroup>& groups = gs.groups;
    const Task* tasks = gs.tasks.p;
    const double* Dsh = nullptr;
    int K = basis_.K;
    const unsigned char* active = d_active_.p;
    if (dthr > 0.0 && !dpairs_host_.empty()) {
        const DPair* pr = d_pairs_.p;
        int np = (int)dpairs_host_.size();
        double* out = d_dsh_.p;
        void* prm[] = {&pr, &np, &Dk, &Dk2, &out};
        sk.kernel(0, density_blocks_spec(np), prm);
        Dsh = d_dsh_.p;
    }
    // float copies of the densities for the FP32 groups' block digestion
    const float *Dj32 = nullptr, *Dk32 = nullptr, *Dk232 = nullptr;
    bool any32 = false;
    for (const auto& g : groups) any32 = any32 || (g.fp32 && g.n > 0);
    if (any32) {
        long long n = nmat();
        d_d32_.alloc((size_t)3 * n);
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
            float* out = d_d32_.p + (size_t)s * n;
            void* prm[] = {&in, &out, &n};
            sk.kernel(0, to_float_spec(n), prm);
            dst[s] = out;
        }
        Dj32 = dst[0];
        Dk32 = dst[1];
        Dk232 = dst[2];
    }
    int* ctr = counters ? counters : d_counters_.p;
    sk.zero(0, ctr, sizeof(int) * std::max<size_t>(1, groups.size()));
    sk.fork();
    // warp groups (the long ones) on the main lane, small classes spread over
    // the others (running the FP32 warp groups on a lane of their own, beside
    // the FP64 ones, measured slower: the persistent grids contend for SMs)
    const int naux = (int)aux_.size();
    int next_aux = 0;
    for (size_t gi = 0; gi < groups.size(); ++gi) {
        const LaunchGroup& g = groups[gi];
        if (g.n == 0) continue;
        KernelSpec ks;
        if (g.kind == 0) {
            const int lane = 1 + next_aux;
            next_aux = (next_aux + 1) % naux;
            if (g.fp32) {
                SmallArgs<float> a{d_pairs_.p, d_rec32_.p, tasks + g.off, (int)g.n, d_boys32_.p,
                                   opt_.screening_threshold, d_qbf_.p, K, Dj, Dk, Dk2, J, Kx, Kx2, Dsh, dthr, active,
                                   Dj32, Dk32, Dk232, d_qbf32_.p};
                cuda_check(small_spec_f32(g.pcb, g.pck, nk, (int)g.n, &ks), "small-class kernel");
                void* prm[] = {&a};
                sk.kernel(lane, ks, prm);
            } else {
                SmallArgs<double> a{d_pairs_.p, d_rec64_.p, tasks + g.off, (int)g.n, d_boys64_.p,
                                    opt_.screening_threshold, d_qbf_.p, K, Dj, Dk, Dk2, J, Kx, Kx2, Dsh, dthr,
                                    active, nullptr, nullptr, nullptr};
                cuda_check(small_spec_f64(g.pcb, g.pck, nk, (int)g.n, &ks), "small-class kernel");
                void* prm[] = {&a};
                sk.kernel(lane, ks, prm);
            }
        } else {
            cuda_check(warp_spec(g.fp32, nk, g.grid, g.warps_per_cta, g.slice, &ks), "warp kernel");
            if (g.fp32) {
                WarpArgs<float> a{d_pairs_.p, d_rec32_.p, d_pct_.p, d_abs_.p, d_kh_.p, d_kl_.p,
                                  tasks + g.off, (int)g.n, ctr + gi, d_boys32_.p,
                                  opt_.screening_threshold, d_qbf_.p, K, Dj, Dk, Dk2, J, Kx, Kx2, g.slice,
                                  g.lane_min_npp,
                                  Dsh, dthr, nullptr, nullptr, active, Dj32, Dk32, Dk232, d_qbf32_.p};
                void* prm[] = {&a};
                sk.kernel(0, ks, prm);
            } else {
                WarpArgs<double> a{d_pairs_.p, d_rec64_.p, d_pct_.p, d_abs_.p, d_kh_.p, d_kl_.p,
                                   tasks + g.off, (int)g.n, ctr + gi, d_boys64_.p,
                                   opt_.screening_threshold, d_qbf_.p, K, Dj, Dk, Dk2, J, Kx, Kx2, g.slice,
                                   g.lane_min_npp,
                                   Dsh, dthr, nullptr, nullptr, active, nullptr, nullptr, nullptr};
                void* prm[] = {&a};
                sk.kernel(0, ks, prm);
            }
        }
    }
    sk.join();
}

void Job::record_stats(int launches) { record_stats_plan(launches, plan(mixed())); }

void Job::record_stats_plan(int launches, const GroupSet& gs)
{
    float ms = 0.f, kms = 0.f;
    cudaEventElapsedTime(&ms, ev0_, ev1_);
    cudaEventElapsedTime(&kms, evk0_, evk1_);
    stats.ms = ms;
    stats.kernel_ms = kms;
    stats.quartets = gs.nquartets;
    stats.quartets_fp32 = gs.quartets32;
    stats.prim_quartets = gs.prims;
    stats.flops_fp64 = gs.flops64;
    stats.flops_fp32 = gs.flops32;
    stats.launches = launches;
}

void Job::fock_rhf_device(const double* dP, double* dG) { fock_rhf_device_ex(dP, dG, mixed(), 0.0); }

// Fock builds run as CUDA graphs after the first eager build of a variant
// (RHF/UHF x plan x screening): the graph replays the accumulator clears, the
// work-queue resets, every class launch on its stream and the symmetrisation,
// reading the density from the job's input buffers and writing its output
// buffers, so a build costs one graph launch plus two device copies.
cudaGraphExec_t Job::graph_for(int nk, bool mixed_plan, double dthr)
{
    if (no_graphs_) return nullptr;
    GraphEntry& g = graphs_[std::make_tuple(nk, mixed_plan, dthr)];
    if (g.exec) return g.exec;
    if (g.eager_runs < 1) return nullptr;   // the first build of a variant runs eagerly
    const size_t n = (size_t)nmat();
    d_gin_.alloc(n);
    d_gout_.alloc(n);
    if (nk == 2) {
        d_gin2_.alloc(n);
        d_gout2_.alloc(n);
        d_gout3_.alloc(n);
    }
    GraphSink gsink(1 + (int)aux_.size());
    if (nk == 1)
        enqueue_rhf(gsink, d_gin_.p, d_gout_.p, mixed_plan, dthr);
    else
        enqueue_uhf(gsink, d_gin_.p, d_gin2_.p, d_gout_.p, d_gout2_.p, d_gout3_.p, mixed_plan, dthr);
    g.exec = gsink.instantiate();
    return g.exec;
}

void Job::clear_graphs()
{
    for (auto& kv : graphs_)
        if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    graphs_.clear();
}

int Job::max_fragment_K() const
{
    int m = 0;
    for (int f = 0; f < frags_.count(); ++f) m = std::max(m, frags_.K(f));
    return m;
}

void Job::enqueue_finish_rhf(OpSink& sk, const double* Jacc, const double* Kacc, double* dG)
{
    const int* fk = d_fk_.p;
    const long long* fm = d_fmoff_.p;
    const unsigned char* act = d_active_.p;
    void* prm[] = {&Jacc, &Kacc, &dG, &fk, &fm, &act};
    sk.kernel(0, finish_rhf_spec(max_fragment_K(), frags_.count()), prm);
}

void Job::enqueue_rhf(OpSink& sk, const double* dP, double* dG, bool mixed_plan, double dthr)
{
    const size_t n = (size_t)nmat();
    sk.zero(0, d_J_.p, n * sizeof(double));
    sk.zero(0, d_K_.p, n * sizeof(double));
    launch_jk(sk, 1, dP, dP, nullptr, d_J_.p, d_K_.p, nullptr, nullptr, mixed_plan, dthr);
    enqueue_finish_rhf(sk, d_J_.p, d_K_.p, dG);
}

void Job::enqueue_uhf(OpSink& sk, const double* dPa, const double* dPb, double* dJ, double* dKa, double* dKb,
                      bool mixed_plan, double dthr)
{
    long long n = nmat();
    sk.zero(0, d_J_.p, (size_t)n * sizeof(double));
    sk.zero(0, d_K_.p, (size_t)n * sizeof(double));
    sk.zero(0, d_K2_.p, (size_t)n * sizeof(double));
    double* dj = d_Dj_.p;
    void* pa[] = {&dPa, &dPb, &dj, &n};
    sk.kernel(0, add_spec(n), pa);
    launch_jk(sk, 2, d_Dj_.p, dPa, dPb, d_J_.p, d_K_.p, d_K2_.p, nullptr, mixed_plan, dthr);
    const double* jp = d_J_.p;
    const double* kp = d_K_.p;
    const double* k2 = d_K2_.p;
    const int* fk = d_fk_.p;
    const long long* fm = d_fmoff_.p;
    const unsigned char* act = d_active_.p;
    void* prm[] = {&jp, &kp, &k2, &dJ, &dKa, &dKb, &fk, &fm, &act};
    sk.kernel(0, finish_uhf_spec(max_fragment_K(), frags_.count()), prm);
}

void Job::fock_rhf_device_ex(const double* dP, double* dG, bool mixed_plan, double dthr)
{
    cuda_check(cudaSetDevice(device_), "cudaSetDevice");
    const size_t n = (size_t)nmat();
    d_J_.alloc(n);
    d_K_.alloc(n);
    cudaGraphExec_t ge = graph_for(1, mixed_plan, dthr);
    cuda_check(cudaEventRecord(ev0_, stream_), "event");
    if (ge) {
        cuda_check(cudaMemcpyAsync(d_gin_.p, dP, n * sizeof(double), cudaMemcpyDeviceToDevice, stream_), "copy in");
        cuda_check(cudaEventRecord(evk0_, stream_), "event");
        cuda_check(cudaGraphLaunch(ge, stream_), "graph launch");
        cuda_check(cudaEventRecord(evk1_, stream_), "event");
        cuda_check(cudaMemcpyAsync(dG, d_gout_.p, n * sizeof(double), cudaMemcpyDeviceToDevice, stream_), "copy out");
    } else {
        cuda_check(cudaEventRecord(evk0_, stream_), "event");
        StreamSink sk = stream_sink();
        enqueue_rhf(sk, dP, dG, mixed_plan, dthr);
        cuda_check(cudaEventRecord(evk1_, stream_), "event");
        ++graphs_[std::make_tuple(1, mixed_plan, dthr)].eager_runs;
    }
    cuda_check(cudaEventRecord(ev1_, stream_), "event");
    cuda_check(cudaStreamSynchronize(stream_), "fock build");
    record_stats_plan((int)plan(mixed_plan).groups.size() + 1, plan(mixed_plan));
}

void Job::fock_rhf_device_scratch(const double* dP, double* dG, double* Jacc, double* Kacc, int* counters)
{
    cuda_check(cudaSetDevice(device_), "cudaSetDevice");
    int K = basis_.K;
    size_t n = (size_t)K * K;
    StreamSink sk = stream_sink();
    cuda_check(cudaEventRecord(ev0_, stream_), "event");
    sk.zero(0, Jacc, n * sizeof(double));
    sk.zero(0, Kacc, n * sizeof(double));
    cuda_check(cudaEventRecord(evk0_, stream_), "event");
    launch_jk(sk, 1, dP, dP, nullptr, Jacc, Kacc, nullptr, counters, mixed(), 0.0);
    cuda_check(cudaEventRecord(evk1_, stream_), "event");
    enqueue_finish_rhf(sk, Jacc, Kacc, dG);
    cuda_check(cudaEventRecord(ev1_, stream_), "event");
    cuda_check(cudaStreamSynchronize(stream_), "fock build");
    record_stats((int)plan(mixed()).groups.size() + 1);
}

void Job::set_launch_shape(const hfx_launch_shape& s)
{
    if (s.small_chunk < 16 || s.small_chunk > 65536 || s.warp_chunk < 16 || s.warp_chunk > (1 << 20) ||
        s.warp_max_warps < 1 || s.warp_max_warps > 8 || s.lane_min_npp < 0)
        throw Error(HFX_ERR_INVALID, "launch shape out of range");
    shape_ = s;
    build_jk_groups(false, gs_fp64_);
    if (mixed()) build_jk_groups(true, gs_mixed_);
    d_counters_.alloc(std::max<size_t>(1, std::max(gs_fp64_.groups.size(), gs_mixed_.groups.size())));
}

// Coordinate search over the launch shape: for each parameter in turn (small
// chunk, warp chunk, warps per CTA, lane-mode threshold), try its candidates with the others held,
// keep the fastest; each trial times the job's own plan (mixed when the job
// is mixed) at density P on the device, the best of `builds` builds.
double Job::autotune_launch_shape(const double* P, int builds, hfx_launch_shape* out)
{
    const size_t n = (size_t)nmat();
    DevBuf<double> dP, dG;
    dP.alloc(n);
    dG.alloc(n);
    cuda_check(cudaMemcpyAsync(dP.p, P, n * sizeof(double), cudaMemcpyHostToDevice, stream_), "H2D P");
    builds = std::max(1, std::min(builds, 10));
    auto trial = [&](const hfx_launch_shape& s) {
        set_launch_shape(s);
        double best = 1e30;
        fock_rhf_device_ex(dP.p, dG.p, mixed(), 0.0);   // first build of the plan (eager)
        for (int b = 0; b < builds; ++b) {
            fock_rhf_device_ex(dP.p, dG.p, mixed(), 0.0);
            best = std::min(best, (double)stats.kernel_ms);
        }
        return best;
    };
    hfx_launch_shape cur = shape_;
    double cur_ms = trial(cur);
    static const int small_c[] = {64, 128, 256, 512, 1024};
    static const int warp_c[] = {1024, 2048, 4096, 8192, 16384};
    static const int wpc_c[] = {2, 4, 8};
    static const int lane_c[] = {0, 6, 12, 24};
    for (int param = 0; param < 4; ++param) {
        const int* c = param == 0 ? small_c : param == 1 ? warp_c : param == 2 ? wpc_c : lane_c;
        const int nc = param == 2 ? 3 : param == 3 ? 4 : 5;
        for (int i = 0; i < nc; ++i) {
            hfx_launch_shape s = cur;
            int& field = param == 0 ? s.small_chunk
                         : param == 1 ? s.warp_chunk
                         : param == 2 ? s.warp_max_warps
                                      : s.lane_min_npp;
            if (field == c[i]) continue;
            field = c[i];
            const double ms = trial(s);
            if (ms < cur_ms * 0.99) {
                cur = s;
                cur_ms = ms;
            }
        }
    }
    set_launch_shape(cur);
    if (out) *out = cur;
    return cur_ms;
}

double Job::autotune_fp32_threshold(const double* P, double target_dE, double* dE_out, double* ms64, double* msmx)
{
    const size_t n = (size_t)nmat();
    std::vector<double> G64(n), Gm(n);
    fock_rhf_ex(P, G64.data(), false, 0.0);
    fock_rhf_ex(P, G64.data(), false, 0.0);
    const double t64 = stats.ms;
    static const double cand[] = {3e-1, 1e-1, 3e-2, 1e-2, 3e-3, 1e-3, 1e-4, 1e-5};
    double best = 0.0, best_dE = 0.0, best_ms = t64;
    const int prec0 = opt_.precision;
    const double tau0 = opt_.fp32_threshold;
    opt_.precision = HFX_PREC_MIXED;
    d_d32_.alloc((size_t)3 * nmat());
    for (double tau : cand) {
        opt_.fp32_threshold = tau;
        build_jk_groups(true, gs_mixed_);
        d_counters_.alloc(std::max<size_t>(1, std::max(gs_fp64_.groups.size(), gs_mixed_.groups.size())));
        fock_rhf_ex(P, Gm.data(), true, 0.0);
        double dE = 0.0;
        for (size_t i = 0; i < n; ++i) dE += P[i] * (Gm[i] - G64[i]);
        dE *= 0.5;
        if (std::fabs(dE) <= target_dE) {
            fock_rhf_ex(P, Gm.data(), true, 0.0);
            best = tau;
            best_dE = dE;
            best_ms = stats.ms;
            break;
        }
    }
    if (best > 0.0) {
        opt_.fp32_threshold = best;
        build_jk_groups(true, gs_mixed_);
    } else {
        opt_.precision = prec0;
        opt_.fp32_threshold = tau0;
        if (mixed()) build_jk_groups(true, gs_mixed_);
    }
    d_counters_.alloc(std::max<size_t>(1, std::max(gs_fp64_.groups.size(), gs_mixed_.groups.size())));
    if (dE_out) *dE_out = best_dE;
    if (ms64) *ms64 = t64;
    if (msmx) *msmx = best_ms;
    return best;
}

void Job::fock_uhf_device(const double* dPa, const double* dPb, double* dJ, double* dKa, double* dKb)
{
    fock_uhf_device_ex(dPa, dPb, dJ, dKa, dKb, mixed(), 0.0);
}

void Job::fock_uhf_device_ex(const double* dPa, const double* dPb, double* dJ, double* dKa, double* dKb,
                             bool mixed_plan, double dthr)
{
    cuda_check(cudaSetDevice(device_), "cudaSetDevice");
    const size_t n = (size_t)nmat();
    d_J_.alloc(n);
    d_K_.alloc(n);
    d_K2_.alloc(n);
    d_Dj_.alloc(n);
    cudaGraphExec_t ge = graph_for(2, mixed_plan, dthr);
    cuda_check(cudaEventRecord(ev0_, stream_), "event");
    if (ge) {
        const size_t b = n * sizeof(double);
        cuda_check(cudaMemcpyAsync(d_gin_.p, dPa, b, cudaMemcpyDeviceToDevice, stream_), "copy in");
        cuda_check(cudaMemcpyAsync(d_gin2_.p, dPb, b, cudaMemcpyDeviceToDevice, stream_), "copy in");
        cuda_check(cudaEventRecord(evk0_, stream_), "event");
        cuda_check(cudaGraphLaunch(ge, stream_), "graph launch");
        cuda_check(cudaEventRecord(evk1_, stream_), "event");
        cuda_check(cudaMemcpyAsync(dJ, d_gout_.p, b, cudaMemcpyDeviceToDevice, stream_), "copy out");
        cuda_check(cudaMemcpyAsync(dKa, d_gout2_.p, b, cudaMemcpyDeviceToDevice, stream_), "copy out");
        cuda_check(cudaMemcpyAsync(dKb, d_gout3_.p, b, cudaMemcpyDeviceToDevice, stream_), "copy out");
    } else {
        cuda_check(cudaEventRecord(evk0_, stream_), "event");
        StreamSink sk = stream_sink();
        enqueue_uhf(sk, dPa, dPb, dJ, dKa, dKb, mixed_plan, dthr);
        cuda_check(cudaEventRecord(evk1_, stream_), "event");
        ++graphs_[std::make_tuple(2, mixed_plan, dthr)].eager_runs;
    }
    cuda_check(cudaEventRecord(ev1_, stream_), "event");
    cuda_check(cudaStreamSynchronize(stream_), "fock build");
    record_stats_plan((int)plan(mixed_plan).groups.size() + 2, plan(mixed_plan));
}

void Job::fock_rhf(const double* P, double* G) { fock_rhf_ex(P, G, mixed(), 0.0); }

void Job::fock_rhf_ex(const double* P, double* G, bool mixed_plan, double dthr)
{
    cuda_check(cudaSetDevice(device_), "cudaSetDevice");
    size_t n = (size_t)nmat();
    d_D_.alloc(n);
    d_out1_.alloc(n);
    cuda_check(cudaMemcpyAsync(d_D_.p, P, n * sizeof(double), cudaMemcpyHostToDevice, stream_), "H2D");
    fock_rhf_device_ex(d_D_.p, d_out1_.p, mixed_plan, dthr);
    cuda_check(cudaMemcpyAsync(G, d_out1_.p, n * sizeof(double), cudaMemcpyDeviceToHost, stream_), "D2H");
    cuda_check(cudaStreamSynchronize(stream_), "D2H");
}

void Job::fock_uhf(const double* Pa, const double* Pb, double* J, double* Ka, double* Kb)
{
    fock_uhf_ex(Pa, Pb, J, Ka, Kb, mixed(), 0.0);
}

void Job::fock_uhf_ex(const double* Pa, const double* Pb, double* J, double* Ka, double* Kb, bool mixed_plan,
                      double dthr)
{
    cuda_check(cudaSetDevice(device_), "cudaSetDevice");
    size_t n = (size_t)nmat();
    d_D_.alloc(n);
    d_D2_.alloc(n);
    d_out1_.alloc(n);
    d_out2_.alloc(n);
    d_out3_.alloc(n);
    cuda_check(cudaMemcpyAsync(d_D_.p, Pa, n * sizeof(double), cudaMemcpyHostToDevice, stream_), "H2D");
    cuda_check(cudaMemcpyAsync(d_D2_.p, Pb, n * sizeof(double), cudaMemcpyHostToDevice, stream_), "H2D");
    fock_uhf_device_ex(d_D_.p, d_D2_.p, d_out1_.p, d_out2_.p, d_out3_.p, mixed_plan, dthr);
    cuda_check(cudaMemcpyAsync(J, d_out1_.p, n * sizeof(double), cudaMemcpyDeviceToHost, stream_), "D2H");
    cuda_check(cudaMemcpyAsync(Ka, d_out2_.p, n * sizeof(double), cudaMemcpyDeviceToHost, stream_), "D2H");
    cuda_check(cudaMemcpyAsync(Kb, d_out3_.p, n * sizeof(double), cudaMemcpyDeviceToHost, stream_), "D2H");
    cuda_check(cudaStreamSynchronize(stream_), "D2H");
}

void Job::eri_unique(double thr, double* out)
{
    cuda_check(cudaSetDevice(device_), "cudaSetDevice");
    if (frags_.count() != 1) throw Error(HFX_ERR_INVALID, "eri_unique: packed job");
    size_t P = (size_t)basis_.K * (basis_.K + 1) / 2;
    size_t nq = P * (P + 1) / 2;
    DevBuf<double> d_out;
    d_out.alloc(nq);
    cuda_check(cudaMemsetAsync(d_out.p, 0, nq * sizeof(double), stream_), "memset");
    std::vector<Task> tasks;
    int maxacc, maxw, maxr;
    // every quartet whose shell-level bound can pass the BF-level test
    build_tasks(thr, tasks, maxacc, maxw, maxr);
    DevBuf<Task> dt;
    dt.upload(tasks, stream_);
    LaunchArgs a = base_args();
    a.thr = thr;
    a.eri = d_out.p;
    run_eri_tasks(dt, (int)tasks.size(), maxacc, maxw, maxr, a);
    cuda_check(cudaMemcpyAsync(out, d_out.p, nq * sizeof(double), cudaMemcpyDeviceToHost, stream_), "D2H");
    cuda_check(cudaStreamSynchronize(stream_), "eri_unique");
}

}  // namespace hfx
