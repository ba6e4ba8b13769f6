/*
 * cbx.h -- C ABI of the GB300 (sm_103a) GBLUP / ssGBLUP engine.
 *
 * Each entry point replaces one piece of the CosmicBLUP CPU path (the
 * reference file:line it stands in for is given beside it).  Conventions:
 *
 *  - plain C: opaque handle, int32 status (CBX_OK == 0), no exceptions cross
 *    the boundary; cbx_last_error(h) returns the message of the last failure;
 *  - one CUDA stream per handle; a handle is not thread-safe (the reference is
 *    driven from one host thread too);
 *  - matrices are dense column-major FP64 unless stated (Eigen's default
 *    storage); symmetric matrices are stored in full;
 *  - every buffer argument is HOST memory unless the name ends in "_dev".
 *
 * There is no CPU fallback: if the CUDA runtime or an sm_103a device is not
 * available, cbx_create fails with CBX_ERR_CUDA.
 */
#ifndef CBX_H_
#define CBX_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  CBX_OK = 0,
  CBX_ERR_ARG = 1,         /* invalid argument (std::invalid_argument in the reference) */
  CBX_ERR_CUDA = 2,        /* CUDA runtime / library failure */
  CBX_ERR_FORMAT = 3,      /* malformed input file bytes (bad BED magic, truncated, ...) */
  CBX_ERR_TIMEOUT = 4,     /* a device-side wait gave up (bounded spin) */
  CBX_ERR_BREAKDOWN = 5,   /* breakdown where the caller cannot continue (PCG itself returns its
                              iterate, as the reference does) */
  CBX_ERR_NONFINITE = 6,   /* NaN / Inf in inputs or iterates */
  CBX_ERR_NOTCONV = 7,     /* iteration limit reached where the caller needs convergence (PCG
                              itself returns its iterate and true residual, as the reference) */
  CBX_ERR_FACTOR = 8,      /* dense factorization failed (not positive definite) */
  CBX_ERR_STATE = 9,       /* call order violated (e.g. solve before upload) */
  CBX_ERR_UNSUPPORTED = 10 /* option the GPU path does not implement */
};

typedef struct cbx_handle cbx_handle;

/* ---- lifetime ----------------------------------------------------------- */
int cbx_create(int device, cbx_handle** out);
int cbx_destroy(cbx_handle* h);
const char* cbx_last_error(const cbx_handle* h);
int cbx_version(void);                                /* 10000*major + 100*minor + patch */
/* Kernel launches issued by this handle since creation (for benchmarks). */
int64_t cbx_launch_count(const cbx_handle* h);
/* Synchronize the handle's stream. */
int cbx_sync(cbx_handle* h);

/* ---- PLINK BED statistics ------------------------------------------------
 * Replaces the per-SNP stats pass of GrmBuilder::compute
 * (src/core/grm_builder.cpp:175-263) on top of PlinkReader::openBed's checks
 * (src/core/plink_reader.cpp:66-91).  bed points at the whole .bed file
 * (3-byte magic included), bed_bytes is its size.  Outputs (length m, int32):
 * observed calls, sum of allele-1 copies, counts of codes 00 / 10 / 11.
 * Any output pointer may be NULL. */
int cbx_bed_snp_counts(cbx_handle* h, const uint8_t* bed, int64_t bed_bytes,
                       int64_t n, int64_t m, int32_t* n_obs, int32_t* sum_x,
                       int32_t* n_hom1, int32_t* n_het, int32_t* n_hom2);

/* ---- Genotype matrix-free products ---------------------------------------
 * cbx_geno_attach replaces PlinkReader::openBed + computeStats
 * (src/core/plink_reader.cpp:66-91, 186-237): the payload of the whole .bed file
 * (bed_bytes, magic included) is copied to the device once and kept in the handle
 * for the products below.  Per SNP: mean = sum of the observed codes' allele-1
 * counts / observed calls, p = mean / 2, var = 2p(1-p), inv_std = 1 / sqrt(var),
 * or 0 when var < 1e-9 or nothing is observed (bit-identical to the reference's
 * FP64 arithmetic).  means / inv_stds (length m) may be NULL. */
int cbx_geno_attach(cbx_handle* h, const uint8_t* bed, int64_t bed_bytes, int64_t n, int64_t m,
                    double* means, double* inv_stds);
/* Y (m x nvec, column-major) = Z^T V (V: n x nvec), Z_ij = (x_ij - mean_j) inv_std_j
 * for an observed call and 0 for a missing one: PlinkReader::multiply_Zt_v
 * (src/core/plink_reader.cpp:341-392).  Sums are exact in 64-bit fixed point (one
 * rounding of each input below 2^-62 of sum|v|); CBX_ERR_NONFINITE for NaN / Inf. */
int cbx_geno_zt_v(cbx_handle* h, int32_t nvec, const double* V, double* Y);
/* Y (n x nvec) = Z V (V: m x nvec), each term first rounded to float as the
 * reference's per-SNP val_map is: PlinkReader::multiply_Z_v
 * (src/core/plink_reader.cpp:239-293).  SNPs with inv_std = 0 are skipped. */
int cbx_geno_z_v(cbx_handle* h, int32_t nvec, const double* V, double* Y);
/* SNP-effect back-solve of the result writer (src/solve/result_writer.cpp:565-623,
 * the --bfile branch): q = G^-1 u_g, effect_j = ((Z^T q)_j / inv_std_j) / total_2pq
 * (0 when inv_std_j = 0), freq_j = mean_j / 2, total_2pq = sum of var_j >= 1e-9.
 * G^-1 is Ginv (host, n_g x n_g) when given, else the handle's device inverse
 * (cbx_invert_psd) or its dense Q^-1 (cbx_mme_set_qinv_dense) of order n_g;
 * otherwise CBX_ERR_STATE ("Could not locate Ginv for back-solving").
 * n_g must equal the attached sample count.  freq / total_2pq may be NULL. */
int cbx_snp_effects(cbx_handle* h, const double* u_g, int64_t n_g, const double* Ginv,
                    double* effect, double* freq, double* total_2pq);

/* ---- Genomic relationship matrix -----------------------------------------
 * Replaces GrmBuilder::compute(const PlinkReader&) for algorithm 1 (VanRaden)
 * with one population, no SNP weights and no HWE filter
 * (src/core/grm_builder.cpp:63-405; accessors getGrm / getSum2pq /
 * getTotalSnps / getAlleleFreqs, src/core/grm_builder.h:51-58).
 *   min_maf     : GrmBuilder::Options::min_maf (0.01f by default)
 *   algorithm   : must be 1 (others return CBX_ERR_UNSUPPORTED)
 *   block_size  : GrmBuilder::Options::block_size; only changes the order in
 *                 which sum 2pq is accumulated, exactly as the reference does
 * Outputs (each may be NULL):
 *   G           : n*n FP64, G = Z Z^T / sum_2pq
 *   xx_counts   : n*n int32, sum over MAF-valid SNPs of x_i x_k (missing = 0),
 *                 the exact integer cross-products formed on the tensor cores
 *   allele_freqs: m floats, (float)freq or -1 for filtered SNPs
 *   sum2pq, n_valid: scalars
 * G is also kept on the device inside the handle (see cbx_invert_psd). */
int cbx_grm_bed(cbx_handle* h, const uint8_t* bed, int64_t bed_bytes, int64_t n,
                int64_t m, float min_maf, int algorithm, int64_t block_size,
                double* G, int32_t* xx_counts, float* allele_freqs,
                double* sum2pq, int64_t* n_valid);

/* ---- Relationship-matrix files ---------------------------------------------
 * cbx_write_upper_packed writes the device GRM (which = 0, from cbx_grm_bed) or the
 * device G^-1 (which = 1, from cbx_invert_psd) as a COSMIC_UPPER_PACKED file
 * (io::write_upper_packed_binary, src/core/upper_packed_binary.cpp:27-68, as called
 * by write_matrix_bin, src/core/matrix_io.cpp:479-484): the 60-byte header, then
 * A(i, j) for i <= j column by column in FP64.  cbx_write_grm_gcta writes the device
 * GRM as GrmBuilder::save does (src/core/grm_builder.cpp:1873-1922): .grm.bin holds
 * G(i, j) for j <= i row by row as float, .grm.N.bin the same layout filled with
 * (float)n_valid.  The .id files (sample names) stay with the caller. */
int cbx_write_upper_packed(cbx_handle* h, int32_t which, const char* path);
int cbx_write_grm_gcta(cbx_handle* h, const char* bin_path, const char* n_path, int64_t n_valid);

/* ---- Text result files -----------------------------------------------------
 * GSOutput::writeResults (src/solve/result_writer.cpp:64-430) for one genetic
 * component, tag "GA" (GBLUP), "HA" (ssGBLUP) or "PA" (pedigree); numbers in the
 * default C++ stream format (6 significant digits), as the reference writes them.
 * No GPU is involved.
 *  cbx_write_vars: Item / Var / Var_SE / h2 / h2_SE / h2_Pr(Chisq) rows for the
 *    component and "e" (h2 SEs by the delta method, Pr = erfc((h2/se)/sqrt 2)).
 *  cbx_write_beta: Levels / Estimation / SE per fixed-effect column (names[p]);
 *    beta_se NULL writes "nan".
 *  cbx_write_rand: ID / tag / residuals / n_obs per animal (q animals, ids[q] or
 *    NULL for "UNK_<k>"): the mean over its records of u and of y - Xb - u and
 *    its record count, animals in order of first record, then the others sorted
 *    by ID with their solution u and "nan" residual.  Records and design as
 *    cbx_mme_create. */
int cbx_write_vars(const char* path, const char* tag, double var_u, double se_u, double var_e, double se_e);
int cbx_write_beta(const char* path, int64_t p, const char* const* names, const double* beta,
                   const double* beta_se);
int cbx_write_rand(const char* path, const char* tag, int64_t n_rec, const double* y, const int32_t* aid,
                   const int64_t* fx_ptr, const int32_t* fx_col, const double* fx_val, int64_t p,
                   const double* beta, int64_t q, const double* u, const char* const* ids);

/* ---- Mixed-model equations (one random component) ------------------------
 * Replaces MMELHSBuilder::initialize / build_lhs / build_rhs
 * (src/core/mme_builder.cpp:72-387, header src/core/mme_builder.h:26-71).
 * Records follow GenRecord (src/core/design.h:20-27): y, aid = 1-based row of
 * Qinv (0 = no random effect); the fixed-effect design follows
 * FixedDesignG::rows (src/core/design.h:32-38) in CSR form: record i owns
 * (fx_col[k], fx_val[k]) for fx_ptr[i] <= k < fx_ptr[i+1], columns < p.
 * The LHS is [X'X X'Z; Z'X Z'Z + lambda Qinv]; lambda is given per solve. */
int cbx_mme_create(cbx_handle* h, int64_t n_rec, int64_t p, int64_t q, const double* y,
                   const int32_t* aid, const int64_t* fx_ptr, const int32_t* fx_col,
                   const double* fx_val);

/* on != 0: an MME created later with the same p and q keeps the previous MME's
 * last data solution and probe solutions as the starting points of its solves
 * (the reference keeps last_solution across the iterations of one run,
 * src/core/vce.cpp:1226-1235); a later cbx_mme_set_qinv_* keeps them too.
 * Residual carries to a new lambda and the gradient's forward state are
 * dropped, since they belong to the old operator.  Off by default: every MME
 * then starts cold, and its results do not depend on earlier MMEs. */
int cbx_mme_keep_warm(cbx_handle* h, int32_t on);

/* Qinv dense, q x q (DenseMatrixAdapter, src/core/matrix_adapter.h:116-153).
 * Qinv == NULL takes the inverse left on the device by cbx_invert_psd. */
int cbx_mme_set_qinv_dense(cbx_handle* h, const double* Qinv, int64_t q);

/* Qinv = A + S Gd S^T: A sparse q x q in CSR (a_ptr[q+1] int64, a_col int32,
 * a_val), Gd dense ng x ng, gmap[k] = row of Qinv for dense row k
 * (SplitMatrixAdapter, src/core/matrix_adapter.h:232-373, with the G^-1 and
 * A22^-1 blocks pre-combined into Gd = G^-1 - A22^-1).  Gd == NULL with ng > 0
 * uses the block that cbx_ssgblup_qinv left on the device of this handle
 * (CBX_ERR_STATE when there is none of order ng). */
int cbx_mme_set_qinv_split(cbx_handle* h, const int64_t* a_ptr, const int32_t* a_col,
                           const double* a_val, const double* Gd, int64_t ng,
                           const int32_t* gmap);

/* Solve LHS(lambda) X = B for nrhs right-hand sides (column-major dim x nrhs,
 * dim = p + q).  Replaces PCGSolver::solve with the block-Jacobi
 * preconditioner (src/core/pcg_solver.h:60-128, 436-536); all right-hand sides
 * share each matrix read.  use_x0: X holds the initial guess.
 * tol_mode 0: stop on ||r||/||b|| < tol (recursive residual, the reference);
 * tol_mode 1: stop on ||r|| < tol (MatrixFreePCG, src/core/matrix_free_pcg.h:51).
 * precision 0: FP64 throughout; 1: FP32 PCG bulk with iterative refinement
 * in FP64, stopping on the true residual b - A x: recomputed in FP64, or,
 * once a correction d is below 2^-8 of x, updated as r -= A d with a
 * float-float block product (error below that of an FP64 b - A x).
 * iters / relres (length nrhs, may be NULL) receive CG iterations and the
 * final relative residual.  As PCGSolver::solve (pcg_solver.h:482-495, 530-534),
 * neither the iteration limit nor a breakdown (|p'Ap| < 1e-300 again after one
 * restart from p = z) is an error: the column keeps its last iterate, iters gets
 * maxit and relres its true residual ||b - A x|| / ||b|| (0 when b = 0).
 * CBX_ERR_NONFINITE for a NaN / Inf iterate. */
int cbx_pcg_solve(cbx_handle* h, double lambda, int32_t nrhs, const double* B, double* X,
                  int32_t use_x0, double tol, int32_t maxit, int32_t tol_mode,
                  int32_t precision, int32_t* iters, double* relres);

/* Y = Qinv X for nrhs column-major q-vectors (AbstractMatrix::operator*,
 * src/core/matrix_adapter.h:19). */
int cbx_qinv_apply(cbx_handle* h, int32_t nrhs, const double* X, double* Y);

/* ---- Kernel timing (no reference counterpart: benchmark instrumentation) ---
 * When enabled, every launch of the dense block product (the G^-1 / H^-1 part
 * of the MME operator) is bracketed by CUDA events on the handle's stream.
 * cbx_profile_read sums, for bucket 0 (FP32 launches) or 1 (FP64 launches),
 * the launch count, their device time and their algorithmic bytes (the dense
 * block once plus the gathered vectors and outputs).  Bucket 2 holds the GRM
 * kernel of cbx_grm_bed, its "bytes" being the algorithmic integer operations
 * 2 n^2 m_valid.  Enabling clears the log.  cbx_timer_start / cbx_timer_stop
 * bracket any sequence of calls with CUDA events on the handle's stream. */
int cbx_profile_enable(cbx_handle* h, int32_t on);
int cbx_profile_read(cbx_handle* h, int32_t bucket, int64_t* launches, double* total_ms,
                     double* total_bytes);
int cbx_timer_start(cbx_handle* h);
int cbx_timer_stop(cbx_handle* h, double* ms);
/* Named NVTX range around a sequence of calls on this thread, so that a profiler
 * can select the kernels launched inside it; no effect without a profiler. */
int cbx_range_push(const char* name);
int cbx_range_pop(void);

/* ---- Pinned host buffers (no reference counterpart) ------------------------
 * Page-locks / releases a caller's host buffer (cudaHostRegister), so that the
 * host <-> device copies of the entry points above run at the link's full rate
 * instead of through pageable staging.  Optional; CBX_ERR_CUDA if the range cannot
 * be registered. */
int cbx_host_register(void* p, int64_t bytes);
int cbx_host_unregister(void* p);

/* ---- Launch-shape autotuner (no reference counterpart) ---------------------
 * Kernels with several launch shapes that give bit-identical results (the
 * float-float block product's piece width and rows per warp, the single-RHS GEMV's
 * rows per warp and loads in flight, the genotype products' chunking) time each
 * shape once per (kernel, device, size class, width) on the live operands and keep
 * the fastest (a shape must beat the default by 1.5 %).  Tuning never changes a
 * result.  It is on unless the environment sets CBX_TUNE=0; cbx_tune_enable
 * switches it process-wide, cbx_tune_reset forgets every decision, and
 * cbx_tune_report writes one line per decision (kernel, device, size classes,
 * width, chosen shape, measured ms per shape) into buf (cap bytes, NUL-ended). */
int cbx_tune_enable(int32_t on);
int cbx_tune_reset(void);
int cbx_tune_report(char* buf, int64_t cap);

/* ---- G inverse with eigen-bending -----------------------------------------
 * Replaces invert_psd_matrix (src/core/matrix_io.cpp:488-501): eigenvalues
 * below max(1e-12 lambda_max, 1e-6) are raised to that bound, then
 * U diag(1/lambda) U^T, in FP64.  M == NULL inverts the GRM left on the device
 * by cbx_grm_bed.  The inverse stays on the device (use it with
 * cbx_mme_set_qinv_dense(h, NULL, n)); Minv (host, n x n) may be NULL. */
int cbx_invert_psd(cbx_handle* h, const double* M, int64_t n, double ridge, double* Minv);

/* ---- Pedigree: Henderson A^-1 and the ssGBLUP H^-1 blocks ----------------
 * cbx_ainv_henderson replaces genmatrix::ml + the Henderson A^-1 assembly
 * (src/core/a_matrix.cpp:127-186, 392-439): dam / sire are 0-based parent
 * indices (-1 or out of range = unknown).  Call with ptr == NULL to get *nnz,
 * then with ptr (n + 1), col / val (nnz) to receive the upper+lower CSR of A^-1.
 * F (inbreeding) and dii_out (Mendelian sampling variances) may be NULL. */
int cbx_ainv_henderson(cbx_handle* h, int64_t n, const int64_t* dam, const int64_t* sire,
                       int64_t* nnz, int64_t* ptr, int32_t* col, double* val, double* F,
                       double* dii_out);

/* cbx_ssgblup_qinv replaces MatrixBuilder's H^-1 path (src/io/
 * relationship_builder.cpp:495-584): A22 = rows/columns gmap of A (by the
 * T D T' recursion over generations on the device; parents must precede
 * progeny), optional tuneG (tune_g != 0), Gb = (1 - alpha) G* + alpha A22,
 * Gd = tau Gb^-1 (eigen-bending) - omega A22^-1, and installs
 * Qinv = A^-1 + S Gd S' on the MME (q = n) as cbx_mme_set_qinv_split would.
 * G == NULL uses the device GRM of this handle (order ng).  A22_out / Gd_out
 * (ng x ng) may be NULL.  Gd stays on the device for later MMEs of the handle
 * (cbx_mme_set_qinv_split with Gd == NULL). */
int cbx_ssgblup_qinv(cbx_handle* h, int64_t n, const int64_t* dam, const int64_t* sire, int64_t ng,
                     const int32_t* gmap, const double* G, double alpha, int32_t tune_g, double tau,
                     double omega, double ridge, double* A22_out, double* Gd_out);

/* ---- AI-REML, one random component ---------------------------------------
 * Mirrors VCEConfig (src/core/vce.h:140-165) with the defaults of Config
 * (src/config/config.h:41-57): ai_maxit 20, vce_tol 1e-4, vce_mc_samples 100,
 * pcg_maxit 10000, pcg_tol 1e-10. */
typedef struct cbx_reml_config {
  int32_t max_iter;      /* REML iterations */
  double tol;            /* stop when |d var_u| + |d var_e| < tol */
  int32_t mc_samples;    /* Hutchinson samples parameter (min 30 / max 100 at 100) */
  int32_t pcg_max_iter;  /* per PCG solve */
  double pcg_tol;        /* relative residual of every PCG solve */
  int32_t precision;     /* 0: FP64 PCG, 1: FP32 PCG + FP64 refinement */
  int32_t mode;          /* 0: dense exact AI when dim < 5000, else EM + Hutchinson
                            (run_ai_iteration's choice); 1: EM; 2: dense exact;
                            3: data-driven AI (run_aireml_step, src/core/vce.cpp:2414-2857)
                            with the LHS factored on the device (dim <= 24,576): exact
                            tr(Qinv C^uu), AI_ij = 1/2 v_i'P v_j from two extra solves,
                            Newton step with up to 15 logL-checked halvings; EM when the
                            step fails or no factorization fits, as the reference does
                            without a direct solver */
  int32_t seed;          /* probe seed (AdaptiveTraceEstimator default 42) */
} cbx_reml_config;

/* Diagnostics of one REML iteration. */
typedef struct cbx_reml_iter_info {
  int32_t kind;          /* 0: EM + Hutchinson, 1: dense exact AI, 2: data-driven AI */
  double var_u, var_e;   /* variances after the iteration */
  double logL;           /* REML log-likelihood (dense exact step; calc_logL_internal at the
                            accepted point for the data-driven AI step), NaN otherwise */
  double trace;          /* tr(Qinv C^uu): Hutchinson estimate (EM), exact (data-driven AI) */
  int32_t probes;        /* probe vectors used */
  int64_t pcg_iters;     /* CG iterations over all solves of the iteration */
  int64_t matvecs;       /* operator applications (one matrix read each) */
  double e_sse, uQu;     /* e'e and u'Qinv u of the data solve (EM) */
} cbx_reml_iter_info;

void cbx_reml_config_default(cbx_reml_config* cfg);

/* One AI-REML iteration on the MME of this handle: run_ai_iteration
 * (src/core/vce.cpp:1334-1660) restricted to its single-component branches:
 * run_dense_exact_step (:2949-3195) or the EM update with Hutchinson traces
 * (:1490-1574).  var_u / var_e are updated in place; info may be NULL. */
int cbx_reml_iterate(cbx_handle* h, const cbx_reml_config* cfg, double* var_u, double* var_e,
                     cbx_reml_iter_info* info);

/* Full AI_REML::solve loop (src/core/vce.cpp:741-837).  history (length
 * max_iter) and solution (length dim: the last data solve) may be NULL. */
int cbx_reml_solve(cbx_handle* h, const cbx_reml_config* cfg, double* var_u, double* var_e,
                   int32_t* iterations, int32_t* converged, double* solution,
                   cbx_reml_iter_info* history);

/* ---- Batched independent GBLUP problems ----------------------------------
 * Many uneven GBLUP problems -- each one GrmBuilder::compute + the eigen-bent
 * invert_psd_matrix + AI_REML::solve, i.e. one reference run (the reference
 * runs them one after the other) -- share one GPU: nworkers host threads each
 * own a handle (one stream, its own library handles and buffers, reused from
 * problem to problem) and take problems largest first, so the streams of
 * small problems overlap on the GPU.  Every problem gets exactly the
 * single-problem path (results equal the per-problem calls).  Each problem's
 * status code lands in its result; the call returns the first non-zero one
 * (CBX_OK when all succeeded). */
typedef struct cbx_batch_problem {
  const uint8_t* bed;        /* PLINK BED (with its 3-byte header), bed_bytes long */
  int64_t bed_bytes, n, m;   /* n animals = q, m SNPs */
  int64_t n_rec, p;          /* records, fixed-effect columns */
  const double* y;           /* n_rec */
  const int32_t* aid;        /* n_rec, 1-based row of G^-1 (0 = none) */
  const int64_t* fx_ptr;     /* fixed-effect design CSR (as cbx_mme_create) */
  const int32_t* fx_col;
  const double* fx_val;
  double var_u, var_e;       /* starting variances */
} cbx_batch_problem;

typedef struct cbx_batch_result {
  int32_t status;            /* CBX_OK or the failing call's code */
  int32_t iterations, converged;
  double var_u, var_e;
  int64_t pcg_iters;         /* CG iterations over the whole REML run */
  double seconds;            /* wall time of this problem on its worker */
  double* solution;          /* caller-owned, length p + n, or NULL */
} cbx_batch_result;

int cbx_batch_reml(int device, int32_t nprob, const cbx_batch_problem* probs, float min_maf,
                   const cbx_reml_config* cfg, int32_t nworkers, cbx_batch_result* results);

/* ---- Final MME solve and fixed-effect standard errors ---------------------
 * Replaces GSSolve::solve (src/solve/mixed_model_solver.cpp:37-420) for one
 * random component: lambda = var_e / var_u (0 if var_u <= 1e-9), sol (dim) =
 * C^-1 W'y; with calc_se, beta_se[i] = sqrt(max(0, var_e (C^-1)_ii)) and
 * Cinv_beta (p x p) from p unit right-hand sides solved as one block.
 * solver 0: dense Cholesky when Qinv is dense and dim < 10000 (the reference's
 * direct path), otherwise as 1; 1: PCG, relative tolerance; 2: PCG, absolute
 * tolerance, warm-started from the last REML data solve (the matrix-free path,
 * :239-256).  beta_se / Cinv_beta may be NULL. */
int cbx_final_solve(cbx_handle* h, double var_u, double var_e, int32_t solver, double tol,
                    int32_t maxit, int32_t precision, int32_t calc_se, double* sol, double* beta_se,
                    double* Cinv_beta);

/* ---- Multi-trait GBLUP ----------------------------------------------------
 * cbx_mt_vce replaces MvEigenVce (src/core/eigen_vce.cpp:106-266) as GSVce
 * runs it (src/variance/variance_estimator.cpp:86-325, projection on):
 * Y (n x t, column-major, complete cases), X (n x p, column-major dense
 * fixed-effect design), G (n x n) or NULL for G = (G^-1)^-1 from the device
 * G^-1 of this handle (cbx_invert_psd).  Projection onto null(X'), eigen-
 * decomposition of the projected G, then EM on Vg / Ve (t x t, row-major)
 * from Cov(Y)/2 until both relative Frobenius changes are below tol (the
 * reference uses max_iter = max(500, 25 vce_max_iter), tol = vce_tol).
 * 1 <= t <= 8, n <= 46,000.  CBX_ERR_FACTOR if some V_i is not positive
 * definite (the reference throws). */
int cbx_mt_vce(cbx_handle* h, int64_t n, int32_t t, int64_t p, const double* Y, const double* X,
               const double* G, int32_t max_iter, double tol, double* Vg, double* Ve,
               int32_t* iterations, int32_t* converged);

/* cbx_mt_solve replaces GSSolve::solveMultiTrait (src/solve/
 * mixed_model_solver.cpp:425-524): the explicit Kronecker MME
 * [Ve^-1 (x) X'X, Ve^-1 (x) X'; Ve^-1 (x) X, Ve^-1 (x) I + Vg^-1 (x) G^-1]
 * with right-hand side [Ve^-1 (x) X' ; Ve^-1 (x) I] vec(Y), built on the device
 * and solved by dense Cholesky.  Ginv (n x n) or NULL for the device G^-1.
 * beta (p t) and u (n t) come back trait-major (index trait * p + effect,
 * trait * n + animal).  (n + p) t <= 46,000. */
int cbx_mt_solve(cbx_handle* h, int64_t n, int32_t t, int64_t p, const double* Y, const double* X,
                 const double* Ginv, const double* Vg, const double* Ve, double* beta, double* u);

/* ---- REML gradient (backward entry) --------------------------------------
 * d logL / d (var_u, var_e) in grad[2], as the data-driven AI-REML score of
 * run_aireml_step (src/core/vce.cpp:2648-2675):
 *   grad_u = (u'Qinv u + var_e tr - q var_u) / (2 var_u^2)
 *   grad_e = (e'e - var_e (n - p - q + lambda tr)) / (2 var_e^2)
 * tr = tr(Qinv C^uu) is estimated from nprobe Rademacher probes (the
 * reference's stream: batches of 16 from mt19937_64(seed + done)) solved as
 * multi-RHS blocks (64 columns in mixed precision, 32 in FP64), or computed exactly from the
 * q unit vectors when exact_trace != 0.  precision as cbx_pcg_solve.
 * The entry is the backward pass of cbx_reml_iterate: when the handle's last EM
 * iteration (or gradient call) started at exactly (var_u, var_e) with the same seed,
 * precision and pcg_tol, its data-solve terms and the z'Qinv C^uu z values of the
 * probes it solved are reused; only probes beyond those are solved, from their stored
 * solutions of the previous call (true residuals carried to the new lambda in mixed
 * precision).  Right after an EM iteration with nprobe <= its probe count no solve runs
 * (*pcg_iters == 0).  Otherwise the data solve starts from the last data solution.
 * The trace sum and the score are formed on the device.
 * trace / pcg_iters may be NULL. */
int cbx_reml_gradient(cbx_handle* h, double var_u, double var_e, int32_t nprobe, int32_t seed,
                      int32_t exact_trace, int32_t precision, double pcg_tol, int32_t pcg_maxit,
                      double* grad, double* trace, int64_t* pcg_iters);
/* One REML iteration (as cbx_reml_iterate) followed by the REML gradient at its
 * starting point from nprobe probes (as cbx_reml_gradient with cfg's seed,
 * precision and PCG settings).  In the EM branch with mixed precision the
 * gradient's first probes (up to 79, whole 16-probe batches) join the
 * iteration's data + probe block, so one multi-RHS solve serves both; the
 * iteration's estimator still uses exactly the probes its stopping rule
 * selects.  grad (2) gets the score; info, trace, grad_pcg_iters (CG
 * iterations of the gradient's own solves) and solution (dim: the last data
 * solve, as cbx_reml_solve returns it) may be NULL. */
int cbx_reml_iterate_grad(cbx_handle* h, const cbx_reml_config* cfg, int32_t nprobe, double* var_u,
                          double* var_e, cbx_reml_iter_info* info, double* grad, double* trace,
                          int64_t* grad_pcg_iters, double* solution);
/* REML log-likelihood by dense Cholesky of the LHS (dim <= 24,576): with a dense
 * Qinv, run_dense_exact_step's compute_logL (src/core/vce.cpp:2974-3007); with a
 * split Qinv (ssGBLUP), calc_logL_internal (:3533-3588), which omits the constant
 * log|A| (it does not depend on the variances). */
int cbx_reml_logl_dense(cbx_handle* h, double var_u, double var_e, double* logL);

/* ---- Dense Qinv product without device allocation -------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory while they run (a host framework that owns the whole device memory
 * pool; latency-critical loops that must not call cudaMalloc / cudaFree, which
 * may synchronize the device): Y = Qd X for the dense Qinv of the handle's MME
 * (cbx_mme_set_qinv_dense), X and Y column-major q x nrhs DEVICE arrays.  Every
 * intermediate lives in one static 32 MiB device array (resident on each GPU
 * that loads the library until the process exits): q is limited to about 65,000
 * (CBX_ERR_ARG beyond).  A handle's first call resolves that array's address and
 * should come before any stream capture; calls that overlap on the GPU share the
 * array and race.  Runs on the handle's stream; the result agrees within rounding
 * with cbx_qinv_apply's (the two sum in different orders). */
int cbx_dense_apply_noalloc(cbx_handle* h, int32_t nrhs, const double* X_dev, double* Y_dev);

#ifdef __cplusplus
}
#endif
#endif /* CBX_H_ */
