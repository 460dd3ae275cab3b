// hfx_device.cuh -- device-side data layout and helpers shared by the
// shell-quartet kernels.
//
// HBM layout of one job (all arrays device-resident for the job's lifetime):
//   DPair[npairs]    one record per shell pair (A >= B in shell order), the
//                    shell with the higher L stored first ("0" side)
//   pp_geo[npp]      PairGeo per primitive pair: (p, Px, Py, Pz)
//   E pool           per primitive pair, the dense Hermite->Cartesian matrix
//                    E[ab][tuv] (n0*n1 x H(l0+l1)), with the primitive weights
//                    w_i(a) w_j(b) (coefficient x cart_norm) and
//                    exp(-mu |AB|^2) folded in; tuv in the reference's packed
//                    order (integrals.hpp:343-358)
//   Qbf[K(K+1)/2]    BF-level Schwarz bounds, pair_index order
//   boys table       F_m(T_k), T_k = k/16, m = 0..kBoysM-1
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace hfx {

// Launch configuration of one kernel: the stream path hands it to
// cudaLaunchKernel, the graph path to cudaGraphAddKernelNode.
struct KernelSpec {
    const void* func = nullptr;
    dim3 grid, block;
    size_t smem = 0;
};

constexpr int kBoysM = 20;          // orders stored (12 + 7 Taylor terms + 1)
constexpr int kBoysInvStep = 16;    // grid step 1/16
constexpr int kBoysTMax = 36;       // table covers [0, 36]; upward recursion beyond
constexpr int kBoysN = kBoysTMax * kBoysInvStep + 1;
// FP32 kernels read their own Boys table, one 8-float row per (L, k):
// {F_L, F_{L+1}, F_{L+2}/2, F_{L+3}/6, F_{L+4}/24, exp(-T_k), 0, 0} at T_k =
// k/16 (the Taylor terms of F_L about T_k pre-scaled), for L <= kBoys32MaxL,
// so that one evaluation is two 16-byte loads.
constexpr int kBoys32MaxL = 12;
constexpr int kBoys32Row = 8;
// The FP64 Fock kernels' table, one 8-double row per (L, k): {F_L, F_{L+1},
// F_{L+2}/2!, ..., F_{L+6}/6!, exp(-T_k)} at T_k = k/16, L <= kBoys64MaxL:
// the 7-term Taylor expansion of F_L about T_k with its coefficients
// pre-scaled (four 16-byte loads and six FMAs, no multiplies).
constexpr int kBoys64MaxL = 12;
constexpr int kBoys64Row = 8;

// Primitive-pair geometry: p = alpha + beta and the product centre P.
struct __align__(32) PairGeo {
    double p, x, y, z;
};
__host__ __device__ inline PairGeo make_pairgeo(double p, double x, double y, double z)
{
    PairGeo g;
    g.p = p;
    g.x = x;
    g.y = y;
    g.z = z;
    return g;
}

struct __align__(16) DPair {
    int bf0, bf1;      // first basis function of shell 0 / shell 1
    int l0, l1;        // l0 >= l1
    int pp0, npp;      // primitive-pair range
    long long e_off;   // offset of the first dense E block (elements)
    int same;          // shell 0 == shell 1
    int id;            // pair id (index in the pair array)
    double qmax;       // max_ab sqrt((ab|ab)) over the pair's BF pairs
    long long rec_off; // offset of the first primitive-pair record (elements)
    int pc;            // pair class l0*(l0+1)/2 + l1
    int sh0, sh1;      // shell indices of shell 0 / shell 1 within the pair's molecule
    // A packed job holds several molecules: the pair's basis-function and
    // shell indices are local to its molecule, whose K x K matrices start at
    // element moff of the packed D/J/K buffers (row stride kdim) and whose
    // BF-pair Schwarz table starts at qoff.  A single-molecule job has
    // frag = 0, pbase = 0, moff = qoff = 0 and kdim = K.
    int kdim;          // basis functions of the pair's molecule
    int pbase;         // pair id of the molecule's first shell pair
    int frag;          // molecule index
    long long moff;    // first element of the molecule's matrices in the packed buffers
    long long qoff;    // first element of the molecule's BF-pair Schwarz bounds
};

// Triangular index of a shell pair (the pair array's order).
__host__ __device__ inline int shell_pair_id(int a, int b)
{
    return a > b ? a * (a + 1) / 2 + b : b * (b + 1) / 2 + a;
}

// Primitive-pair record of the class kernels, for a pair of class (l0, l1):
//   [p, Px, Py, Pz, 1/p, c_0 ... c_{ncoef-1}] padded to an even length, where the
// c_k are the structurally non-zero Hermite->Cartesian coefficients
//   c = w_i(a) w_j(b) E^x_{ax bx, t} E^y_{ay by, u} E^z_{az bz, v}
// (weights = contraction coefficient x cart_norm, exp(-mu AB^2) included),
// ordered by component pair ab (a outer), then t, u, v nested.
struct PairClassTab {
    int nab;       // component pairs
    int ncoef;     // coefficients per record
    int stride;    // record length (elements)
    int ab_off;    // offset of this class's ab_start table
    int k_off;     // offset of this class's per-coefficient tables
};
constexpr int kNumPairClasses = 10;
// shared-memory header of the warp kernel (index tables), bytes
constexpr int kWarpSmemHeader = 11776;   // (00) (10) (11) (20) (21) (22) (30) (31) (32) (33)

__host__ __device__ constexpr int dncart(int l) { return (l + 1) * (l + 2) / 2; }
__host__ __device__ constexpr int dnherm(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }

// packed Hermite index of (t,u,v), the reference's packed_r_index_cpu
// (integrals.hpp:343-358): s-major, then t, then u.
__host__ __device__ inline int herm_index(int t, int u, int v)
{
    int s = t + u + v;
    int off = s * (s + 1) * (s + 2) / 6;
    // sum_{aa<t} (s - aa + 1) = t*(s+1) - t*(t-1)/2
    off += t * (s + 1) - t * (t - 1) / 2;
    return off + u;
}

// One unit of work: a shell quartet (bra pair, ket pair), restricted to the
// bra primitive pairs [i0, i1) and the ket primitive pairs [k0, k1).  A
// quartet's primitive quartets can be split into any such tiles, each
// digested on its own (J and K are linear in the integrals): heavily
// contracted quartets are split so that no thread or warp carries a
// disproportionate share of a launch, and launch groups with few quartets
// are split further so that they still fill the GPU.  16 bytes, one vector
// load.
struct __align__(16) Task {
    int bra, ket;
    unsigned short i0, i1, k0, k1;
};
__host__ __device__ inline Task make_task(int bra, int ket, int i0, int i1, int k0, int k1)
{
    Task t;
    t.bra = bra;
    t.ket = ket;
    t.i0 = (unsigned short)i0;
    t.i1 = (unsigned short)i1;
    t.k0 = (unsigned short)k0;
    t.k1 = (unsigned short)k1;
    return t;
}

// Arguments of the unique-ERI kernel (hfx_kernels.cu).
struct LaunchArgs {
    const DPair* pairs;
    const PairGeo* pp_geo;
    const double* epool;
    const double* boys;      // [kBoysN][kBoysM]
    const Task* tasks;
    int ntasks;
    int* counter;            // work-queue head (zeroed before launch)
    int K;
    double thr;              // BF-level Schwarz threshold (< 0: none)
    const double* Qbf;
    double* eri;             // packed unique ERIs, eri_index order
};

// Arguments of the small-class (thread-per-shell-quartet) kernels.
template <typename T>
struct SmallArgs {
    const DPair* pairs;
    const T* rec;
    const Task* tasks;
    int ntasks;
    const T* boys;
    double thr;
    const double* Qbf;
    int K;
    const double* Dj;
    const double* Dk;
    const double* Dk2;
    double* J;
    double* Kx;
    double* Kx2;
    const double* Dsh;         // per shell pair max |D| (density screening), or null
    double dthr;               // skip a quartet when Q_AB Q_CD max|D| < dthr (0: never)
    const unsigned char* active;   // packed jobs: per molecule, 0 = skip its quartets (null: all)
    // FP32 kernels: float copies of Dj / Dk / Dk2 for the block digestion
    const float* Dj32;
    const float* Dk32;
    const float* Dk232;
    // FP32 kernels: float copy of the BF-pair Schwarz bounds (the digestion's
    // screen then needs no FP64 arithmetic); addressed with bra.qoff
    const float* Qbf32;
};

// Arguments of the warp-per-shell-quartet kernel.
template <typename T>
struct WarpArgs {
    const DPair* pairs;
    const T* rec;              // primitive-pair records
    const PairClassTab* pct;   // per pair class
    const int* ab_start;       // per class: nab+1 offsets into the record coefficients
    const short* k_herm;       // per coefficient: packed Hermite index of (t,u,v)
    const short* k_lin;        // per coefficient: t*169+u*13+v, bit 14 = parity of t+u+v
    const Task* tasks;
    int ntasks;
    int* counter;
    const T* boys;             // per-L rows: kBoys64Row doubles (FP64) / kBoys32Row floats (FP32)
    double thr;
    const double* Qbf;
    int K;
    const double* Dj;
    const double* Dk;
    const double* Dk2;
    double* J;
    double* Kx;
    double* Kx2;
    int slice;                 // per-warp shared-memory slice, in T elements
    int lane_min_npp;          // lane-parallel R for L <= 6 and ket npp >= this (0: never)
    const double* Dsh;         // per shell pair max |D| (density screening), or null
    double dthr;               // skip a quartet when Q_AB Q_CD max|D| < dthr (0: never)
    double* Qout_bf;           // Schwarz pass (NK = 0): BF-pair bounds out
    unsigned long long* Qout_sh;   // Schwarz pass: per shell pair max bound (double bits)
    const unsigned char* active;   // packed jobs: per molecule, 0 = skip its quartets (null: all)
    // FP32 kernels: float copies of Dj / Dk / Dk2 for the block digestion
    const float* Dj32;
    const float* Dk32;
    const float* Dk232;
    // FP32 kernels: float copy of the BF-pair Schwarz bounds (the digestion's
    // screen then needs no FP64 arithmetic); addressed with bra.qoff
    const float* Qbf32;
};

#ifdef __CUDACC__
// float -> double by bit manipulation on the integer pipes (exact for normal
// floats; zeros and denormals give a signed zero, infinities and NaNs keep
// their class).  The FP32 kernels convert their digestion sums this way
// before the FP64 atomics, since a conversion instruction runs on the FP64
// pipe, which on this GPU is 1/64 of the FP32 rate.
__device__ __forceinline__ double f32_to_f64_bits(float v)
{
    const unsigned u = __float_as_uint(v);
    const unsigned e = (u >> 23) & 0xffu;
    const unsigned sign = u & 0x80000000u;
    const unsigned m = u & 0x7fffffu;
    const unsigned hi_exp = e == 255u ? 0x7ff00000u : ((e + 896u) << 20);
    const unsigned hi = e == 0u ? sign : (sign | hi_exp | (m >> 3));
    const unsigned lo = e == 0u ? 0u : (m << 29);
    return __hiloint2double((int)hi, (int)lo);
}

// Nearest Boys-table grid point of T (0 <= T < 2^18): k = round(16 T) and the
// Taylor step nd = k/16 - T, without conversion instructions (adding 1.5 * 2^23
// leaves round(16 T) in the float's low mantissa bits).
__device__ __forceinline__ float boys_grid_offset(float T, int& k)
{
    const float magic = 12582912.0f;
    const float t = fmaf(T, (float)kBoysInvStep, magic);
    k = __float_as_int(t) - __float_as_int(magic);
    return (t - magic) * (1.0f / (float)kBoysInvStep) - T;
}

// Digestion atomics: FP64 accumulators, FP32 sums converted on the integer pipes.
template <typename T>
__device__ __forceinline__ void add_to_fp64(double* p, T v)
{
    if constexpr (sizeof(T) == 8)
        atomicAdd(p, v);
    else
        atomicAdd(p, f32_to_f64_bits(v));
}

// Density-weighted Schwarz test of a quartet: the largest density block its
// J and K contributions touch (AB, CD, AC, AD, BC, BD) times Q_AB Q_CD.
__device__ __forceinline__ bool density_negligible(const DPair& b, const DPair& k, const double* Dsh, double dthr)
{
    if (dthr <= 0.0) return false;
    const double* D = Dsh + b.pbase;
    double d = fmax(Dsh[b.id], Dsh[k.id]);
    d = fmax(d, D[shell_pair_id(b.sh0, k.sh0)]);
    d = fmax(d, D[shell_pair_id(b.sh0, k.sh1)]);
    d = fmax(d, D[shell_pair_id(b.sh1, k.sh0)]);
    d = fmax(d, D[shell_pair_id(b.sh1, k.sh1)]);
    return b.qmax * k.qmax * d < dthr;
}

// Digestion form of the FP64 kernels: false = 6 atomics per integral,
// true = per-quartet block sums (the FP32 kernels always use block sums).
// Block sums measured 0-4% slower for FP64 builds (benzene/cc-pVDZ,
// n-decane/6-31G*), which are bound by the FP64 pipe, not by atomics.
constexpr bool kBlockDigestFP64 = false;

// The density the block digestion multiplies with: FP64 kernels the FP64
// matrix, FP32 kernels its float copy.
template <typename T>
__device__ __forceinline__ const T* density_of(const double* d64, const float* d32)
{
    if constexpr (sizeof(T) == 8)
        return d64;
    else
        return d32;
}

// The BF-pair Schwarz bounds a kernel of precision T screens with: FP64
// kernels the double table, FP32 kernels its float copy.
template <typename T, typename A>
__device__ __forceinline__ const T* schwarz_of(const A& a)
{
    if constexpr (sizeof(T) == 8)
        return a.Qbf;
    else
        return a.Qbf32;
}

// Quartet of a molecule that takes no part in this build of a packed job.
__device__ __forceinline__ bool molecule_inactive(const DPair& b, const unsigned char* active)
{
    return active != nullptr && __ldg(active + b.frag) == 0;
}
#endif

}  // namespace hfx
