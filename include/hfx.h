/*
 * hfx.h -- C ABI of libhfx, the GB300 (sm_103a) direct-SCF Fock-build engine
 * for the McMurchie-Davidson Hartree-Fock code KLYYCYNN/hartree_fock_cpp.
 *
 * The engine replaces the reference's ERI call and its per-iteration Fock
 * contraction:
 *   - std::vector<double> ERI_GPU(const std::vector<basis_function>&, double)
 *       declared include/scf.hpp:41-44, defined cuda/src/eri.cu:20-89
 *       -> hfx_eri_unique / hfx_eri_gpu (same packed eri_index layout)
 *   - schwarz_bounds (include/integrals.hpp:732-752)      -> hfx_schwarz
 *   - repulsion_matrix (include/linalg.hpp:100-129)       -> hfx_fock_rhf
 *   - coulomb_matrix + 2x exchange_matrix
 *       (include/linalg.hpp:215-296, called scf.hpp:542-544) -> hfx_fock_uhf
 *   - rhf_diis / uhf_diis with eri_device "GPU"
 *       (include/scf.hpp:205-419 / 423-682)              -> hfx_rhf_diis / hfx_uhf_diis
 * J and K are built directly from shell-quartet ERIs; the ERI tensor is never
 * stored (only hfx_eri_unique, the literal ERI_GPU replacement, writes it).
 *
 * Conventions: all matrices are K x K, row-major, double, in the reference's
 * basis-function order (atoms -> CSV shells -> Cartesian components with lx
 * outer, ly inner, as basis.hpp:52-64).  Buffers are caller-owned host memory
 * unless a function name ends in _device.  Every function returns an
 * hfx_status; no C++ exception crosses this boundary.  A job handle is used by
 * one host thread at a time.  Errors never terminate the process (the
 * reference calls std::exit from cuda_check, cuda/src/eri.cu:8-14).
 */
#ifndef HFX_H
#define HFX_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int hfx_status;

enum {
    HFX_OK = 0,
    HFX_ERR_INVALID = 1,      /* bad argument, size or option */
    HFX_ERR_BASIS = 2,        /* basis file missing / malformed / unsupported element or L */
    HFX_ERR_CUDA = 3,         /* CUDA runtime error (message in hfx_last_error) */
    HFX_ERR_OOM = 4,          /* device or host allocation failed / admission refused */
    HFX_ERR_UNSUPPORTED = 5,  /* feature outside the engine's limits (e.g. L > 3) */
    HFX_ERR_NOT_CONVERGED = 6,/* SCF reached max iterations (results still filled) */
    HFX_ERR_CANCELLED = 7,    /* served job cancelled */
    HFX_ERR_TIMEOUT = 8,      /* served job or bounded device wait timed out */
    HFX_ERR_NUMERIC = 9       /* NaN/Inf in energy or Fock matrix */
};

/* Precision of the Fock build. */
enum {
    HFX_PREC_FP64 = 0,        /* every quartet in FP64 (the all-FP64 oracle path) */
    HFX_PREC_MIXED = 1        /* quartets with Schwarz bound < fp32_threshold in FP32 */
};

/* Density step of the device SCF (hfx_scf_options.eigensolver). */
enum {
    HFX_EIG_AUTO = 0,         /* SP2 projector on the device, syevd fallback */
    HFX_EIG_SYEVD = 1         /* cuSOLVER syevd every iteration */
};

/* ---- basis descriptions -------------------------------------------------- */

/* Basis-function level description: exactly the reference's
 * std::vector<basis_function> (include/types.hpp:16-29) flattened.
 * Consecutive functions must form complete Cartesian shells in
 * angmom_partition order (which basis_construction always produces). */
typedef struct {
    int K;                    /* number of basis functions */
    const double *centres;    /* 3*K, bohr */
    const int *lmn;           /* 3*K, (lx, ly, lz) */
    const int *prim_offset;   /* K+1, range of each function's primitives */
    const double *alpha;      /* exponents */
    const double *coeff;      /* contraction coefficients */
    const double *norm;       /* primitive norms (cart_norm, basis.hpp:28-49) */
} hfx_functions;

/* Molecule + basis-set name, built like basis_construction (basis.hpp:157-262). */
typedef struct {
    int natom;
    const char *const *symbols;  /* element symbols, e.g. "O" */
    const double *xyz;           /* 3*natom, bohr */
    const char *basis_set;       /* "STO-3G", "6-31G", "6-31G*", "cc-pVDZ", "cc-pVTZ" */
    const char *basis_path;      /* directory holding <set>/<El>.csv; NULL = bundled sets */
} hfx_molecule;

/* Engine options (zero-initialise, then set; 0 selects the default). */
typedef struct {
    double screening_threshold; /* BF-level Schwarz cut Q_ij*Q_kl < thr -> 0; default 1e-8
                                   (run.hpp:46 / integrals.hpp:771); set < 0 for no screening */
    int precision;              /* HFX_PREC_FP64 (default) or HFX_PREC_MIXED */
    double fp32_threshold;      /* mixed: shell-quartet bound below this runs in FP32; default 1e-7 */
    int device;                 /* CUDA device ordinal; default 0 */
    int reserved[8];
} hfx_options;

typedef struct hfx_job hfx_job;

/* Build a job from a basis-function list (drop-in for the reference's
 * std::vector<basis_function>).  Uploads pair data, computes the Schwarz
 * table on the device, and builds the screened shell-quartet work lists. */
hfx_status hfx_create(const hfx_functions *basis, const hfx_options *opt, hfx_job **job);

/* Same, building the basis from a molecule and a basis-set name. */
hfx_status hfx_create_molecule(const hfx_molecule *mol, const hfx_options *opt, hfx_job **job);

hfx_status hfx_destroy(hfx_job *job);

/* Number of basis functions of the job. */
hfx_status hfx_nbasis(const hfx_job *job, int *K);

/* Export the job's basis-function list (sizes as in hfx_functions; pass
 * NULL for any array not wanted; nprim_total receives the primitive count). */
hfx_status hfx_export_functions(const hfx_job *job, double *centres, int *lmn, int *prim_offset,
                                double *alpha, double *coeff, double *norm, int *nprim_total);

/* Schwarz bounds Q_ij = sqrt(max((ij|ij),0)) for all K(K+1)/2 pairs in
 * pair_index order (indexing.hpp:33-40); replaces schwarz_bounds
 * (integrals.hpp:732-752). */
hfx_status hfx_schwarz(hfx_job *job, double *Q);

/* RHF two-electron matrix G = J[P] - 1/2 K[P] (linalg.hpp:100-129), P and G
 * K x K host buffers.  Replaces repulsion_matrix(P, ERI). */
hfx_status hfx_fock_rhf(hfx_job *job, const double *P, double *G);

/* UHF: J = J[Pa+Pb], Ka = K[Pa], Kb = K[Pb] (linalg.hpp:215-296). */
hfx_status hfx_fock_uhf(hfx_job *job, const double *Pa, const double *Pb, double *J, double *Ka,
                        double *Kb);

/* Device-pointer variants (K x K double buffers already on the job's device;
 * run on the job's stream, synchronise before returning). */
hfx_status hfx_fock_rhf_device(hfx_job *job, const double *dP, double *dG);
hfx_status hfx_fock_uhf_device(hfx_job *job, const double *dPa, const double *dPb, double *dJ,
                               double *dKa, double *dKb);

/* RHF two-electron matrix like hfx_fock_rhf_device, for callers that cannot
 * allocate device memory at call time (an application whose own allocator
 * owns the GPU memory, or a loop that must not let cudaMalloc synchronise
 * the device).  No counterpart in the reference.  It allocates nothing: its
 * scratch (J/K accumulators, work-queue counters) lives in one static device
 * array of about 4 MB, reserved on a device when the first job is created
 * there (job creation resolves the array's address, which under CUDA's
 * default lazy module loading loads the module holding it) and kept until the
 * process exits.  Limits: K <= 512, else HFX_ERR_UNSUPPORTED.  All
 * calls share the array, so calls that overlap on the GPU race; serialise
 * them.  The job itself must already exist (hfx_create allocates). */
hfx_status hfx_fock_rhf_device_noalloc(hfx_job *job, const double *dP, double *dG);

/* All unique ERIs in the reference's packed layout: out[eri_index(i,j,k,l)],
 * P(P+1)/2 doubles with P = K(K+1)/2, zero where Q_ij*Q_kl < threshold
 * (integrals.hpp:754-787 / cuda/src/eri.cu:20-89). */
hfx_status hfx_eri_unique(hfx_job *job, double threshold, double *out);

/* One-shot literal ERI_GPU(basis, threshold) replacement. */
hfx_status hfx_eri_gpu(const hfx_functions *basis, double threshold, double *out);

/* Statistics of the last Fock build. */
typedef struct {
    double ms;                /* device time of the whole build (CUDA events) */
    double kernel_ms;         /* device time of the shell-quartet kernel launches alone */
    double quartets;          /* surviving shell quartets */
    double quartets_fp32;     /* of which computed in FP32 */
    double prim_quartets;     /* primitive quartets evaluated */
    double flops_fp64;        /* algorithmic flops (MD count) done in FP64 */
    double flops_fp32;        /* algorithmic flops done in FP32 */
    int launches;             /* kernel launches of the build */
    int reserved[7];
} hfx_build_stats;

hfx_status hfx_last_build_stats(const hfx_job *job, hfx_build_stats *stats);

/* Launch shape of a job's Fock-build plans: primitive quartets per task of
 * the thread-per-quartet kernels (small_chunk) and of the warp kernel
 * (warp_chunk; heavily contracted quartets are split into chunks of bra
 * primitive pairs), the warp kernel's maximum warps per CTA (1..8), and the
 * smallest ket primitive-pair count for which the warp kernel computes the
 * R integrals of 32 ket primitive pairs at once, one per lane (L <= 6 only;
 * 0: never; otherwise all lanes work on one primitive pair at a time).
 * Defaults 256 / 4096 / 8 / 6. */
typedef struct {
    int small_chunk;
    int warp_chunk;
    int warp_max_warps;
    int lane_min_npp;
    int reserved[4];
} hfx_launch_shape;

hfx_status hfx_get_launch_shape(const hfx_job *job, hfx_launch_shape *shape);
hfx_status hfx_set_launch_shape(hfx_job *job, const hfx_launch_shape *shape);
/* Autotuner: coordinate search over the four parameters, timing the job's
 * own plan (mixed when the job is mixed) at density P (host K x K) with the
 * best of `builds` device builds per trial; the job keeps the fastest shape.
 * best_ms: its kernel time. */
hfx_status hfx_autotune_launch_shape(hfx_job *job, const double *P, int builds, hfx_launch_shape *shape,
                                     double *best_ms);

/* Autotune the mixed-precision cut for this job: at density P (K*K host, e.g.
 * a converged or near-converged density), build G in FP64 and then in mixed
 * precision for tau = 0.3, 0.1, 0.03, ... 1e-5, keep the largest tau with
 * |1/2 sum P (G_tau - G_fp64)| <= target_dE (Eh) and switch the job to mixed
 * precision at that tau.  tau = 0 if no candidate qualifies (job unchanged).
 * dE / ms_fp64 / ms_mixed (optional) report the chosen tau's energy change and
 * the two build times. */
hfx_status hfx_autotune_fp32_threshold(hfx_job *job, const double *P, double target_dE, double *tau, double *dE,
                                       double *ms_fp64, double *ms_mixed);

/* ---- SCF drivers (scf.hpp semantics) -------------------------------------- */

typedef struct {
    int max_iterations;         /* default 10000 (scf.hpp:213) */
    double epsilon;             /* RMSD(P) and ||FPS-SPF|| threshold; default 1e-6 */
    double damping;             /* default 0.3, first 3 iterations */
    double screening_threshold; /* default 1e-8 */
    double energy_threshold;    /* > 0 adds |E_n - E_{n-1}| < energy_threshold; default off */
    int charge;
    int precision;              /* HFX_PREC_FP64 / HFX_PREC_MIXED */
    double fp32_threshold;      /* mixed precision cut (see hfx_options) */
    int fp64_final_cycles;      /* mixed: once ||FPS-SPF|| < 1000 eps, or when it (below 1e-3) stops falling (no new
                                   low by 10% in four iterations), switch to one full FP64 build and FP64 builds
                                   of the density change (default 0 = on; -1: full FP64 builds instead) */
    int start_diis;             /* default 4 (scf.hpp:235) */
    int max_history;            /* default 8 (scf.hpp:236) */
    int verbose;
    int eigensolver;            /* HFX_EIG_AUTO (0): density of each iteration by the SP2 projector on the device for
                                   K <= 640, cuSOLVER syevd where it does not converge (no HOMO-LUMO gap) and once at
                                   the end for the MO energies and coefficients; HFX_EIG_SYEVD: syevd every iteration */
    int reserved[5];
} hfx_scf_options;

typedef struct {
    double E_tot, E_ele, E_nuc;
    int iterations;
    int converged;
    int K;
    int n_electrons;
    double seconds;             /* wall time of the whole SCF */
    double fock_ms;             /* summed device time of the Fock builds */
    int fock_builds;
    int mixed_builds;           /* builds with FP32 quartets (mixed precision) */
    int fp64_builds;            /* full FP64 builds */
    int delta_builds;           /* FP64 builds of a density change (mixed precision, final cycles) */
    int projections;            /* iterations whose density came from the SP2 projector (device SCF) */
    int projection_fallbacks;   /* iterations where it did not converge and syevd was used */
    int reserved[2];
} hfx_scf_result;

/* RHF (scf.hpp:205-419).  P0: optional K*K initial density (NULL = zero).
 * density / coefficient / mo_energy: optional outputs (K*K, K*K, K). */
hfx_status hfx_rhf_diis(const hfx_molecule *mol, const hfx_scf_options *opt, const double *P0,
                        hfx_scf_result *res, double *density, double *coefficient, double *mo_energy);

/* UHF (scf.hpp:423-682), n_alpha + n_beta electrons. */
hfx_status hfx_uhf_diis(const hfx_molecule *mol, const hfx_scf_options *opt, int n_alpha, int n_beta,
                        const double *Pa0, const double *Pb0, hfx_scf_result *res, double *Pa, double *Pb,
                        double *mo_energy_a, double *mo_energy_b);

/* RHF / UHF SCF on an existing job (its basis, pair data and Schwarz table
 * stay resident; S, H and S^-1/2 are computed once per job).  Same semantics
 * and outputs as hfx_rhf_diis / hfx_uhf_diis; the job's screening and
 * precision options apply, the molecule's charge comes from opt. */
hfx_status hfx_job_rhf(hfx_job *job, const hfx_scf_options *opt, const double *P0, hfx_scf_result *res,
                       double *density, double *coefficient, double *mo_energy);
hfx_status hfx_job_uhf(hfx_job *job, const hfx_scf_options *opt, int n_alpha, int n_beta, const double *Pa0,
                       const double *Pb0, hfx_scf_result *res, double *Pa, double *Pb);

/* The same drivers with a caller-supplied two-electron builder in place of
 * the GPU engine: the host SCF loop (DIIS, eigensolver, convergence logic)
 * can then be checked against another Fock builder, e.g. the reference's
 * stored-tensor contraction.  A builder returns 0 on success. */
typedef int (*hfx_g_builder)(void *user, const double *P, double *G);
typedef int (*hfx_jk_builder)(void *user, const double *Pa, const double *Pb, double *J, double *Ka, double *Kb);
hfx_status hfx_rhf_diis_with_builder(const hfx_molecule *mol, const hfx_scf_options *opt, const double *P0,
                                     hfx_g_builder g, void *user, hfx_scf_result *res, double *density,
                                     double *mo_energy);
hfx_status hfx_uhf_diis_with_builder(const hfx_molecule *mol, const hfx_scf_options *opt, int n_alpha, int n_beta,
                                     hfx_jk_builder jk, void *user, hfx_scf_result *res, double *Pa, double *Pb);

/* Basis-function list of a molecule as the engine builds it (host only, no
 * device work): K, then the hfx_functions arrays (sizes as there; pass NULL
 * to query K and nprim_total first). */
hfx_status hfx_build_functions(const hfx_molecule *mol, int *K, int *nprim_total, double *centres, int *lmn,
                               int *prim_offset, double *alpha, double *coeff, double *norm);

/* Host image of the per-shell-pair data the kernels read (no device work):
 * for each shell pair p: rec[10*p..] = {bf0, bf1, l0, l1, pp0, npp, e_off_lo,
 * e_off_hi, same, id}; geo[4*q..] = (p, Px, Py, Pz) per primitive pair q;
 * epool = the dense E[ab][tuv] blocks.  Query sizes with NULL arrays. */
hfx_status hfx_debug_pair_data(const hfx_molecule *mol, int *npairs, int *nprimpairs, long long *nepool, int *rec,
                               double *geo, double *epool);
/* Test hook (host only, no device work): the shell-pair records of a packed
 * job over n molecules.  Per pair, rec[10*p ..] = frag, kdim, pbase, id, sh0,
 * sh1, bf0, bf1, l0, l1 (shell and function indices local to the molecule)
 * and offs[3*p ..] = moff, qoff, npp.  Pass rec = offs = NULL to get npairs. */
hfx_status hfx_debug_packed_pairs(const hfx_molecule *mols, int n, int *npairs, int *rec, long long *offs);

/* Test hook (no device work): the launch groups of a job's Fock-build plan
 * (mixed != 0: the mixed-precision plan of a mixed job), 10 doubles per
 * group: kind (0 thread-per-quartet class kernel, 1 warp kernel), bra and
 * ket pair class (class kernels), fp32, tasks, algorithmic flops, primitive
 * quartets, grid, shared-memory slice and warps per CTA (warp kernel).
 * Pass rows = NULL to get ngroups.  No counterpart in the reference. */
hfx_status hfx_debug_plan(const hfx_job *job, int mixed, int *ngroups, double *rows);

/* One-electron matrices S, T, V of a molecule (integrals.hpp:10-536), host. */
hfx_status hfx_one_electron(const hfx_molecule *mol, double *S, double *T, double *V, int *K);
/* The same matrices computed on CUDA device `device` (one CTA per shell pair;
 * the SCF entry points use this for their setup).  Host output buffers. */
hfx_status hfx_one_electron_gpu(const hfx_molecule *mol, int device, double *S, double *T, double *V, int *K);

/* ---- request server (continuous batching on one GPU) ---------------------- */

typedef struct hfx_server hfx_server;

typedef struct {
    int max_active;          /* concurrent jobs (worker slots); default 8 */
    double hbm_budget_gb;    /* device memory the jobs may hold; default 80% of free memory */
    int device;
    int precision;           /* default precision of requests (HFX_PREC_*) */
    double fp32_threshold;   /* default mixed-precision cut */
    int pack_max;            /* > 1: packed mode -- each running request joins a Fock session shared
                                with up to pack_max - 1 other requests of the same method, options and
                                size class (K < 100, < 300, larger): every SCF cycle is one build over
                                all of them, one launch per quartet class, and requests that arrive while
                                a session iterates join it at their next cycle; 0 or 1: each request
                                builds on its own streams */
    int reserved[7];
} hfx_server_options;

enum { HFX_JOB_QUEUED = 0, HFX_JOB_RUNNING = 1, HFX_JOB_DONE = 2, HFX_JOB_FAILED = 3 };
/* host-side fault injection (tests): fail the job at this stage */
enum { HFX_FAULT_NONE = 0, HFX_FAULT_SETUP = 1, HFX_FAULT_OOM = 2, HFX_FAULT_ALLOC = 3, HFX_FAULT_ITERATION = 4 };

typedef struct {
    hfx_molecule mol;        /* copied at submission */
    int method;              /* 0 RHF, 1 UHF */
    int n_alpha, n_beta;     /* UHF occupations */
    hfx_scf_options scf;
    int precision;           /* -1: server default */
    double fp32_threshold;   /* 0: server default */
    double timeout_s;        /* 0: none; measured from submission */
    int inject_fault;        /* HFX_FAULT_* (tests) */
    int reserved[7];
} hfx_request;

typedef struct {
    int state;               /* HFX_JOB_* */
    hfx_status status;       /* HFX_OK, HFX_ERR_NOT_CONVERGED or the failure */
    double E_tot;
    int iterations, converged, K;
    double t_submit, t_admit, t_end;   /* steady-clock seconds */
    double fock_ms;
    int fock_builds;
    char message[256];
} hfx_job_info;

typedef struct {
    int queued, running, done, failed, max_concurrent;
    double budget_bytes, in_use_bytes;
    int max_session_members;   /* packed mode: most jobs one Fock session held at once */
    int sessions_created;      /* packed mode: Fock sessions opened so far */
    int reserved[4];
} hfx_server_stats_t;

hfx_status hfx_server_create(const hfx_server_options *opt, hfx_server **server);
hfx_status hfx_server_submit(hfx_server *server, const hfx_request *req, long long *id);
hfx_status hfx_server_poll(hfx_server *server, long long id, hfx_job_info *info);
/* wait for one job (timeout_s <= 0: no limit); HFX_ERR_TIMEOUT if it is still running */
hfx_status hfx_server_wait(hfx_server *server, long long id, double timeout_s, hfx_job_info *info);
hfx_status hfx_server_cancel(hfx_server *server, long long id);
/* wait until the queue is empty and no job runs */
hfx_status hfx_server_drain(hfx_server *server, double timeout_s);
/* converged densities of a finished job (K*K each; Pb for UHF) */
hfx_status hfx_server_density(hfx_server *server, long long id, double *Pa, double *Pb);
hfx_status hfx_server_stats(hfx_server *server, hfx_server_stats_t *stats);
hfx_status hfx_server_destroy(hfx_server *server);

/* ---- lockstep batched SCF (packed Fock builds) ---------------------------
 * Replaces the sequential scan drivers run_bl_scan (run.hpp:300-423) and
 * run_dissociation (run.hpp:498-577), which solve one geometry after another.
 * All n molecules (any mix of sizes and basis sets) share one packed job and
 * iterate in lockstep: each SCF cycle is ONE Fock build over every molecule
 * still iterating (one launch per quartet class over all molecules'
 * quartets, replayed as a CUDA graph), each molecule's O(K^3) SCF steps run
 * on its own stream.  With warm_chain = 0 or 1 every molecule starts from
 * the zero density.  With warm_chain = c > 1 the molecules form chains of c
 * consecutive indices (0..c-1, c..2c-1, ...): inside a chain molecule i
 * starts from molecule i-1's final density, as the reference's sequential
 * scan does from the previous geometry (run.hpp:353-368), so a chain's
 * molecules run one after another while the chains iterate together.
 * One method per batch; UHF takes per-molecule n_alpha[i], n_beta[i].
 * results[i] gets molecule i's result.  HFX_ERR_NOT_CONVERGED if some
 * molecule did not converge (every result still filled); any other failure
 * returns the first failing molecule's status. */
typedef struct {
    int method;              /* 0 RHF, 1 UHF */
    int max_parallel;        /* molecules (chains, with warm_chain > 1) iterating at once (0: all, at most 256) */
    int warm_chain;          /* > 1: warm-started chains of this many consecutive molecules (above) */
    int reserved[5];
} hfx_batch_options;

typedef struct {
    double seconds;          /* wall time of the whole batch, setup included */
    double setup_seconds;    /* bases + packed job (pair data, Schwarz, plans) */
    int cycles;              /* packed Fock builds run */
    int molecules;
    double build_ms;         /* device time of all packed builds */
    double quartets;         /* surviving shell quartets of one packed build, all molecules */
    double flops_fp64;       /* algorithmic FP64 flops of that build */
    double reserved[5];
} hfx_batch_stats;

hfx_status hfx_batch_scf(const hfx_molecule *mols, int n, const int *n_alpha, const int *n_beta,
                         const hfx_scf_options *scf, const hfx_batch_options *opt, hfx_scf_result *results,
                         hfx_batch_stats *stats);

/* ---- electron density and orbitals on grids (cube.hpp:9-168, evaluation.cuh:59-123) ----
 * rho(r) = sum_{mu,nu} P_{mu nu} phi_mu(r) phi_nu(r), psi_i(r) = sum_mu C_{mu i} phi_mu(r)
 * with the basis functions of `basis` (the reference's std::vector<basis_function>,
 * as density_gpu / orbital_gpu take it, visual.cu), on CUDA device `device`.
 * Box grids follow density3d / homo_lumo_3d:
 * res^3 points x_i = (c - L/2) + i (L / (res - 1)) per axis, value of point
 * (i, j, k) at out[(i * res + j) * res + k]; res >= 2.  P and C are K x K
 * row-major host matrices (C's column `column` is the orbital); out is host
 * memory.  Limits: K such that a 32-point tile of all functions fits in
 * shared memory (K <= ~880), at most 32 primitives per shell. */
hfx_status hfx_grid_density(const hfx_functions *basis, int device, const double *P, const double *center, double L,
                            int res, double *rho);
hfx_status hfx_grid_orbital(const hfx_functions *basis, int device, const double *C, int column, const double *center,
                            double L, int res, double *psi);
/* The same at n explicit points (xyz: 3n, bohr): column < 0 evaluates rho
 * with M = P, column >= 0 evaluates psi_column with M = C. */
hfx_status hfx_points_eval(const hfx_functions *basis, int device, const double *M, int column, const double *xyz,
                           long long n, double *out);

/* Last error message of the calling thread (empty if none). */
hfx_status hfx_last_error(char *buf, size_t n);

/* FP64 / FP32 FMA-loop peak of the device, GFLOP/s (roofline denominators). */
hfx_status hfx_measure_peaks(int device, double *fp64_gflops, double *fp32_gflops);
/* FP64 tensor-core (DMMA: mma.sync m8n8k4 f64) loop throughput, GFLOP/s:
 * the ceiling of a tensor-core Hermite->Cartesian transform.  No counterpart
 * in the reference (its transforms are scalar FP64, cuda/include/kernels.cuh:6-80). */
hfx_status hfx_measure_dmma_peak(int device, double *gflops);

#ifdef __cplusplus
}
#endif

#endif /* HFX_H */
