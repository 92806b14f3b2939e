/*
 * qsx — C ABI of the GB300 (sm_103a) Liouville-space propagation library.
 *
 * Every entry point takes caller-owned DEVICE pointers (plain pointers and
 * sizes), an explicit cudaStream_t passed as void*, and returns an int status
 * (QSX_OK = 0).  Nothing is allocated by the library: buffers and scratch
 * ("workspace") come from the caller; qsx_*_workspace_bytes says how much.
 * complex128 arrays are interleaved {re, im} doubles (the layout of
 * torch.complex128 / numpy.complex128), complex64 interleaved floats.
 * No C++ exception crosses this boundary; qsx_last_error_string() describes
 * the last failure on the calling host thread.
 *
 * Each declaration names the reference (whaley-group-berkeley/qspectra)
 * function it replaces, by file:line within that project.
 */
#ifndef QSX_H_
#define QSX_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  QSX_OK = 0,
  QSX_ERR_INVALID_ARG = 1, /* bad shape, size, subspace index or pointer */
  QSX_ERR_CUDA = 2,        /* a CUDA runtime call or launch failed */
  QSX_ERR_UNSUPPORTED = 3, /* valid request the library does not implement */
  QSX_ERR_NONFINITE = 4    /* a NaN/Inf was detected in a state */
};

enum { QSX_FP64 = 0, QSX_FP32 = 1 };

/* Message for the last non-zero status on this host thread. */
const char* qsx_last_error_string(void);

/* Library ABI version (major * 100 + minor). */
int qsx_version(void);

/*
 * One-sided Debye bath correlation function C(x) at n points, complex128 out.
 * Replaces DebyeBath.corr_func_complex (qspectra/bath.py:84-102) with its
 * truncated Matsubara sum of `matsubara_cutoff` terms evaluated in closed
 * form, and Bath.corr_func_real (qspectra/bath.py:17-31) when real_only != 0.
 */
int qsx_debye_corr(const double* x, int64_t n, double temperature,
                   double reorg_energy, double cutoff_freq,
                   int matsubara_cutoff, int real_only, double* out,
                   void* stream);

/*
 * Batched real-symmetric eigensolver (cyclic Jacobi, FP64), n <= 32.
 * H, U: [batch][n][n] row-major; E: [batch][n].  Eigenvalues are sorted
 * ascending inside each diagonal block [block_starts[k], block_starts[k+1])
 * (block_starts is a HOST array of nblocks + 1 ints), which reproduces the
 * g/e/f manifold ordering of Hamiltonian.eig (qspectra/hamiltonian.py:310-328,
 * scipy.linalg.eigh of the non-rotating H).  U holds eigenvectors as columns.
 */
int qsx_eigh_batched(const double* H, int n, int64_t batch, int nblocks,
                     const int* block_starts, double* E, double* U,
                     void* stream);
/* As qsx_eigh_batched; precision QSX_FP32 runs the block Jacobi sweeps of
 * blocks up to 8 states in FP32 (builds that feed FP32 propagation), the
 * outputs still double.  Larger blocks always run in FP64. */
int qsx_eigh_batched_prec(const double* H, int n, int64_t batch, int nblocks,
                          const int* block_starts, int precision, double* E,
                          double* U, void* stream);

/*
 * Redfield operators per disorder sample, FP64.  Replaces redfield_tensor
 * (qspectra/dynamics/redfield.py:9-74) by its exact operator factorisation:
 *   Kt_i = U^T diag(occ_i) U,  Mt_i[c][d] = Kt_i[c][d] * C(E_d - E_c),
 *   GS   = sum_i Kt_i Mt_i      (the eigenbasis Gamma_abbc contraction),
 * with C the Debye correlation function (qsx_debye_corr).  Outputs are
 * scaled by unit_convert.  site_basis != 0 returns G = U GS U^T and
 * M_i = U Mt_i U^T (K_i = diag(occ_i) then needs no output; pass K = NULL);
 * site_basis == 0 returns GS, Mt_i and Kt_i (K must be non-NULL).
 *   E [batch][n], U [batch][n][n], occ [n_sites][n] (shared),
 *   G complex128 [batch][n][n], M complex128 [batch][n_sites][n][n],
 *   K real [batch][n_sites][n][n].  n <= 32, n_sites <= 32.
 * precision QSX_FP64 evaluates everything in FP64; QSX_FP32 evaluates the
 * same formulas in FP32 (for generators that feed the FP32 split-word
 * propagation), with the outputs still stored as complex128 / double.
 */
int qsx_redfield_operators_batched(const double* E, const double* U, int n,
                                   int64_t batch, const double* occ,
                                   int n_sites, double temperature,
                                   double reorg_energy, double cutoff_freq,
                                   int matsubara_cutoff, int discard_imag_corr,
                                   double unit_convert, int site_basis,
                                   int precision, double* G, double* M, double* K,
                                   void* stream);

/*
 * Rotating-frame Hamiltonians of disorder samples: H[s] = base + diag of
 * offsets[s] ([batch][n_sites]) on rows/columns [off, off + n_sites) of the
 * shared n x n base (the site-energy shifts of Hamiltonian.sample,
 * qspectra/hamiltonian.py:552-578).  H [batch][n][n] double.
 */
int qsx_disordered_hamiltonians(const double* base, int n, const double* offsets,
                                int64_t batch, int n_sites, int off, double* H,
                                void* stream);

/*
 * FP64 build for one-exciton Hilbert spaces ('e', 'ge'; 2 <= n_sites <= 8),
 * one warp per sample: the eigendecomposition of the rotating-frame H
 * (Hamiltonian.eig, qspectra/hamiltonian.py:310-328) refined to FP64 from
 * approximate eigenvectors X (two Ogita-Aishima steps R = I - X^T X,
 * S = X^T H X, X <- X + X F, with close pairs finished by FP64 Jacobi
 * rotations), then the site-basis Redfield operators G and M_i of
 * qsx_redfield_operators_batched (site_basis != 0), all in FP64.
 * The coupled block is rows/columns [off, off + n_sites) of each n x n H
 * (n <= 32); states outside it are uncoupled 1 x 1 blocks.  U_approx holds
 * approximate eigenvectors of that block (e.g. from qsx_eigh_batched_prec
 * with QSX_FP32) and may alias U.  Outputs: E [batch][n] (ascending inside
 * the block), U [batch][n][n], G complex128 [batch][n][n], M complex128
 * [batch][n_sites][n][n], scaled by unit_convert, zero outside the block.
 */
int qsx_redfield_build_w64(const double* H, int n, int off, int n_sites,
                           int64_t batch, const double* U_approx,
                           double temperature, double reorg_energy,
                           double cutoff_freq, int matsubara_cutoff,
                           int discard_imag_corr, const double* corr_table,
                           int corr_pieces, double corr_width, double unit_convert,
                           double* E, double* U, double* G, double* M,
                           void* stream);
/*
 * FP32 site-basis Redfield operators for one-exciton Hilbert spaces ('e',
 * 'ge'; 2 <= n_sites <= 8), one warp per sample, from an FP32
 * eigendecomposition (E, U as qsx_eigh_batched_prec with QSX_FP32 stores
 * them).  Same outputs as qsx_redfield_operators_batched with site_basis != 0
 * and QSX_FP32 (redfield_tensor, qspectra/dynamics/redfield.py:9-74, in
 * operator form): with the number-operator couplings of one-exciton states,
 * M_i = Y_i (C Y_i^T), Y_i[a][c] = U[a][c] U[i][c], C[c][d] = C(E_d - E_c),
 * and row i of G is row i of M_i.  The coupled block is rows/columns
 * [off, off + n_sites) of each n x n matrix (n <= 32).  Outputs G complex128
 * [batch][n][n], M complex128 [batch][n_sites][n][n], scaled by
 * unit_convert, zero outside the block.
 */
int qsx_redfield_operators_w32(const double* E, const double* U, int n, int off,
                               int n_sites, int64_t batch, double temperature,
                               double reorg_energy, double cutoff_freq,
                               int matsubara_cutoff, int discard_imag_corr,
                               double unit_convert, double* G, double* M,
                               void* stream);
/* The Matsubara sum S(x) = sum_{k=1}^{K-1} nu_k / ((nu_k^2 - gamma^2)
 * (nu_k - i x)), nu_k = 2 pi k T, of the Debye correlation function
 * (qspectra/bath.py:95-102) as a piecewise Chebyshev table: piece j covers
 * x in [j width, (j + 1) width) with qsx_debye_matsubara_table_degree()
 * complex coefficients, fitted in FP64 to the direct sum; computed on the
 * host into coef (host memory, [pieces][degree] complex128).  The FP64
 * build takes it (device copy) as corr_table, corr_pieces, corr_width and
 * evaluates C(x) there by Clenshaw's recurrence, using the closed form
 * beyond the table or when corr_table is NULL. */
int qsx_debye_matsubara_table(double temperature, double cutoff_freq, int matsubara_cutoff,
                              int pieces, double width, double* coef);
int qsx_debye_matsubara_table_degree(void);

/*
 * Batched dense product C = alpha A B + beta Cin for the third-order
 * engine's many-right-hand-side steps (the t2 integrate over len(t1) states
 * and the einsum('ci,abi') contraction of qspectra/simulate/response.py:
 * 321-336, and the operator transforms and propagator powers behind them).
 * mode 0: real A, B, C; 1: complex A, B, C; 2: complex A, real B; 3: real A,
 * complex B (C complex for modes 1-3).  Complex values are interleaved
 * {re, im}.  A [batch][M][K] row-major with row stride lda and batch stride
 * strideA (0 = shared), likewise B [K][N] and C, Cin [M][N]; strides count
 * elements of the operand's own type.  Cin may be NULL (then beta is
 * ignored) or C itself; C must not alias A or B.  QSX_FP32 runs on the
 * tensor cores (tcgen05, 3xTF32 with FP32 accumulation; status, may be
 * NULL, receives QSX_ERR_CUDA if a completion wait times out), QSX_FP64 on
 * the CUDA cores.  batch <= 65535, K >= 1.
 */
int qsx_gemm_batched(int precision, int mode, int64_t batch, int M, int N, int K,
                     const void* A, int64_t lda, int64_t strideA,
                     const void* B, int64_t ldb, int64_t strideB,
                     const void* Cin, int64_t ldcin, int64_t strideCin, double beta,
                     void* C, int64_t ldc, int64_t strideC, double alpha,
                     int32_t* status, void* stream);

/*
 * Dense Liouvillian block L[idx, idx] (transposed when transpose != 0, the
 * Heisenberg picture).  Replaces RedfieldModel.evolution_super_operator
 * (qspectra/dynamics/redfield.py:95-104, 146-152) sliced by
 * LiouvilleSpaceModel.equation_of_motion (liouville_space.py:316-330):
 *   L[(a,b),(c,d)] = -i uc (H_ac d_bd - d_ac H_db) - s_abcd R_abcd,
 *   R_abcd = d_bd G_ac + d_ac conj(G_bd)
 *          - sum_i (K_i,ac conj(M_i,bd) + M_i,ac K_i,bd),
 * with (a,b) <-> column-stacked index a + n*b, s = secular mask
 * (redfield.py:77-83) when secular != 0 (eigenbasis inputs only) else 1.
 *   H real [n][n] per sample (stride H_stride elements, 0 = shared),
 *   G, M from qsx_redfield_operators_batched, K real [n_sites][n][n] with
 *   stride K_stride (0 = shared); K == NULL means the site-basis number
 *   operators K_i = diag(occ_i) given by occ [n_sites][n] (device),
 *   idx int32 [m] (device), L complex128 [batch][m][m].
 */
int qsx_redfield_liouvillian_batched(const double* H, int64_t H_stride,
                                     const double* G, const double* M,
                                     const double* K, int64_t K_stride,
                                     const double* occ,
                                     int n, int n_sites, int64_t batch,
                                     double unit_convert, const int* idx,
                                     int m, int secular, int transpose,
                                     double* L, void* stream);

/*
 * Liouvillian block and its RK4 propagator in one pass (site basis,
 * non-secular): D = P - I (as qsx_rk4_propagator_batched) of the block
 * L[idx, idx] (transposed when transpose != 0) that
 * qsx_redfield_liouvillian_batched produces with K == NULL, built in shared
 * memory and never written to HBM.  Replaces the same reference code as
 * those two calls (redfield.py:95-104 and 146-152, liouville_space.py:316-330,
 * simulate/utils.py:44-49).  m <= 64; returns QSX_ERR_UNSUPPORTED when the
 * operators plus three m x m tiles exceed 227 KB of shared memory.
 */
int qsx_redfield_propagator_batched(const double* H, int64_t H_stride,
                                    const double* G, const double* M,
                                    const double* occ, int n, int n_sites,
                                    int64_t batch, double unit_convert,
                                    const int* idx, int m, int transpose,
                                    double h, int precision, void* D,
                                    void* stream);

/*
 * K-step blocked propagator for the time loop: from D = P - I (complex64 or
 * complex128 [batch][m][m], as qsx_rk4_propagator_batched returns) build
 * [batch][m + nselect (K - 1)][m]: rows < m hold P^K - I, row
 * m + (k - 1) nselect + q holds row select[q] of P^k - I (1 <= k < K).
 * The same RK4 iterates as the step-by-step loop (simulate/utils.py:44-49),
 * regrouped so qsx_rk4_batched with block_k = K does one matrix-vector pass
 * per K steps.  m <= 64, K <= 64; select int32 [nselect] (device).
 */
int qsx_rk4_block_matrix_batched(const void* D, int m, int64_t batch,
                                 int precision, int K, const int* select,
                                 int nselect, void* out, void* stream);

/*
 * Real form of Hermitian Liouville blocks (no reference counterpart: an
 * exact change of coordinates).  A Redfield generator with a real symmetric
 * Hamiltonian maps Hermitian density matrices to Hermitian ones, so on a
 * diagonal block (n x n states, m = n^2, column-stacked) its RK4 propagator
 * is a real m x m matrix in the coordinates
 *   x[a + n b] = Re rho_ab (a <= b),  Im rho_ba (a > b),
 * with the populations x[a + n a] = rho_aa among them; each step then costs
 * m^2 real multiply-adds instead of m^2 complex ones.
 *
 * qsx_hermitian_real_form: complex [batch][m][m] (complex64 for QSX_FP32,
 * complex128 for QSX_FP64) -> real [batch][m][m] (float / double).
 * qsx_redfield_propagator_hermitian_batched: as
 * qsx_redfield_propagator_batched for the diagonal block of the nb states
 * `states` (Hilbert indices, nb <= 8, m = nb^2), writing the real
 * D_r = P_r - I [batch][m][m].  The real generator is a sparse linear map
 * of the sources [Re B[s]_xy, Im B[s]_xy for s, x, y < nb] ++
 * [uc H_xy for x, y < nb], B[s] = G - sum_i occ_is M_i on the block, given
 * per entry r * m + c as four int32 (16-byte aligned): two 16-bit source
 * indices in each of the first two, four signed 8-bit coefficients in the
 * third, the fourth unused; it depends on nb only and is built once by the
 * caller.
 * qsx_rk4_block_matrix_real_batched: qsx_rk4_block_matrix_batched on real
 * matrices; each sample's (m + nselect (K - 1)) x m output starts at a
 * multiple of 4 values (sample stride = that size rounded up to 4).
 * qsx_rk4_real_block_mean: the K-step blocked loop on FP32 real matrices
 * [batch][m + nselect (K - 1)][m] in that padded layout (m in
 * {9,16,25,36,49,64}, at most 512
 * rows), split-word FP32 state from y0 (double [batch][m], y0_stride 0 =
 * shared); out_mean (double [nsteps + 1][nselect]) is the ensemble mean of
 * the selected coordinates at every step; workspace of
 * qsx_rk4_real_block_workspace_bytes() bytes.  group = samples per CTA
 * (0 = the library's choice, one).  With group <= 1, when the selected
 * rows fit 128 and the block-steps 128, the loop runs in two passes: the
 * state chain (one warp per sample) writes every block-start state into the
 * workspace (batch x (nsteps / K + 1) x 4 ceil(m / 4) floats after the
 * partial sums), then the ensemble contraction runs on the tensor cores
 * (3xTF32 tcgen05 products summed in tensor memory); status also receives
 * QSX_ERR_CUDA if a tensor-core completion wait times out.
 */
int qsx_hermitian_real_form(const void* A, int n, int64_t batch, int precision,
                            void* R, void* stream);
int qsx_redfield_propagator_hermitian_batched(const double* H, int64_t H_stride,
                                              const double* G, const double* M,
                                              const double* occ, int n, int n_sites,
                                              int64_t batch, double unit_convert,
                                              const int* states, int nb,
                                              const int* recipe, double h,
                                              int precision, void* D, void* stream);

/*
 * Rows of complex column-stacked n x n matrices to and from the coordinates
 * of their Hermitian and anti-Hermitian parts (V = V_h + i V_a): merge 0
 * splits in complex [batch][rows][m] into out real [batch][2 rows][m] (the
 * V_h rows, then the V_a rows); merge 1 is the inverse.
 */
int qsx_hermitian_rows(const void* in, int n, int64_t rows, int64_t batch, int precision,
                       int merge, void* out, void* stream);
int qsx_rk4_block_matrix_real_batched(const void* D, int m, int64_t batch,
                                      int precision, int K, const int* select,
                                      int nselect, void* out, void* stream);
/* The same real blocked matrices (FP32) on the tensor cores: each phase is
 * one M = 128 x N = 16 ceil(m/16) x K = 8 ceil(m/8) tcgen05.mma chain in
 * 3xTF32 (hi/lo TF32 split of both operands, FP32 accumulation in tensor
 * memory) computing the next square and the next selected rows together;
 * persistent CTAs, two per SM.  Supported when
 * qsx_rk4_block_matrix_real_tc_supported(m, K, nselect): m <= 64,
 * K = 2^J or 2^J + 1, at most 64 selected rows entering a product.  D
 * [batch][m][m] contiguous, 4-byte aligned; out as for the batched form
 * (per-sample stride rounded up to 4 floats); status (device int, may be
 * NULL) receives QSX_ERR_CUDA if a completion wait times out. */
int qsx_rk4_block_matrix_real_tc_supported(int m, int K, int nselect);
int qsx_rk4_block_matrix_real_tc(const float* D, int m, int64_t batch, int K,
                                 const int* select, int nselect, float* out,
                                 int32_t* status, void* stream);
size_t qsx_rk4_real_block_workspace_bytes(int m, int64_t batch, int K, int nsteps,
                                          int nselect, int group);
int qsx_rk4_real_block_mean(const float* matrix, int m, int64_t batch, int K,
                            int nsteps, const double* y0, int64_t y0_stride,
                            const int* select, int nselect, int group,
                            double* out_mean, void* workspace, size_t workspace_bytes,
                            int32_t* status, void* stream);

/*
 * RK4 propagator D = P - I with P = sum_{k<=4} (hL)^k / k!, i.e. exactly one
 * classical RK4 step of dy/dt = L y (the step inside the integrate loop,
 * qspectra/simulate/utils.py:44-49, with zvode replaced by RK4).
 * L complex128 [batch][m][m]; D complex64 (QSX_FP32) or complex128
 * (QSX_FP64) [batch][m][m].  m <= 64.
 */
int qsx_rk4_propagator_batched(const double* L, int m, int64_t batch,
                               double h, int precision, void* D, void* stream);

/*
 * Batched fixed-step RK4 time loop for linear equations of motion.
 * Replaces integrate / _integrate (qspectra/simulate/utils.py:16-109) for
 * eom(t, y) = L y, and the serial ensemble loop of optional_ensemble_average
 * (qspectra/simulate/decorators.py:40-64) when out_mean is set.
 */
typedef struct {
  int32_t precision;      /* QSX_FP64 or QSX_FP32 (split-word FP32 state) */
  int32_t form;           /* 0: matrix = D = P - I, 1: matrix = L (stages) */
  int32_t m;              /* state dimension */
  int32_t nsteps;         /* RK4 steps */
  int64_t batch;          /* independent samples */
  const void* matrix;     /* complex64/complex128 [batch][m][m] */
  int64_t matrix_stride;  /* elements between samples, 0 = shared */
  double h;               /* step, used by form 1 */
  const double* y0;       /* complex128 [batch][m] */
  int64_t y0_stride;      /* elements between samples, 0 = shared */
  int32_t save_every;     /* output every save_every steps, from step 0 */
  int32_t nproj;          /* rows of proj (dense projections), 0 = none */
  const double* proj;     /* complex128 [nproj][m] per sample */
  int64_t proj_stride;    /* elements between samples, 0 = shared */
  int32_t nselect;        /* selected state components, 0 = none */
  int32_t block_k;        /* > 1: K-step blocked matrix (see below), else 0 */
  const int32_t* select;  /* int32 [nselect] (device) */
  double* out_state;      /* complex128 [batch][nsave][m] or NULL */
  double* out_proj;       /* complex128 [batch][nsave][nout] or NULL */
  double* out_mean;       /* complex128 [nsave][nout] or NULL */
  double mean_scale;      /* out_mean = mean_scale * sum over samples */
  void* workspace;        /* scratch for out_mean partial sums */
  size_t workspace_bytes;
  int32_t* status;        /* device int: set to QSX_ERR_NONFINITE on NaN/Inf */
  int32_t variant;        /* kernel variant, 0 = the planner's choice; with block_k:
                             1 = one thread per matrix row, 2 / 4 = that many lanes
                             per row, 3 / 5 = two rows per thread over two / four
                             lanes (an autotuner times them and passes the
                             fastest) */
  int32_t reserved;       /* must be 0 */
} qsx_rk4_args;
/* nsave = nsteps / save_every + 1; nout = nproj if nproj > 0 else nselect.
 *
 * K-step blocking (block_k = K > 1): `matrix` holds, per sample, the
 * (m + nselect (K - 1)) x m output of qsx_rk4_block_matrix_batched and one
 * matrix-vector pass advances K RK4 steps while still producing the selected
 * components at every step (same iterates y_{n+1} = P y_n, regrouped).
 * Needs QSX_FP32, form 0, nselect outputs only, save_every 1, no out_state,
 * nsteps % K == 0 and m in {9, 16, 25, 36, 49, 64}.  The select entries must
 * be distinct and in [0, m): the blocked kernels check the table on the
 * device and, for a bad one, set QSX_ERR_INVALID_ARG in status and write
 * nothing. */

/* sizeof(qsx_rk4_args) as compiled into the library, for FFI bindings to
 * check their struct declaration against. */
size_t qsx_rk4_args_bytes(void);

int qsx_rk4_workspace_bytes(const qsx_rk4_args* args, size_t* bytes);
int qsx_rk4_batched(const qsx_rk4_args* args, void* stream);

/*
 * Ensemble-mean K-step blocked RK4 loop that allocates nothing (no reference
 * counterpart: an addition for callers that cannot call cudaMalloc, such as
 * a plug-in inside a host application that owns all device memory, or an
 * embedded runtime with a fixed memory budget).  Same arguments and results
 * as qsx_rk4_batched with block_k > 1 and out_mean set, except that
 * `workspace` is ignored: the partial sums live in a 16 MiB device array
 * built into the library, which every GPU that loads the library keeps until
 * the process exits.  Requests whose (nsteps + 1) * nselect * 16 bytes exceed
 * 16 MiB are rejected with QSX_ERR_INVALID_ARG; larger batches run with fewer
 * persistent CTAs so their partial sums fit.  The first call on each device
 * looks up the array's address (cudaGetSymbolAddress) with that device
 * current, so make it before any stream capture; calls outside a capture
 * look it up again, so the address stays right after a device reset.
 * Every call shares the array and clears the part it uses: calls that
 * overlap on the GPU race.
 */
int qsx_rk4_block_mean_noalloc(const qsx_rk4_args* args, void* stream);

/*
 * K-step blocked loop for projected signals of small blocks (m <= 8, up to
 * 4 projections), the time loop of the Heisenberg-picture linear response.
 * qsx_rk4_proj_block_build: from D = P - I (complex64 [batch][m][m]) and the
 * projections proj (complex128 [nproj][m], shared) write, per sample, the
 * complex64 (m + nproj K) x m matrix: rows 0..m-1 = P^K - I, row
 * m + k nproj + p = proj_p P^k (k = 0..K-1).
 * qsx_rk4_proj_block_mean: out_mean (complex128 [nsteps + 1][nproj]) = the
 * ensemble mean over samples of proj_p . y_n with y_{n+1} = P y_n from y0
 * (complex128 [batch][m], y0_stride 0 = shared), nsteps % K == 0; split-word
 * FP32 state; workspace of qsx_rk4_proj_block_workspace_bytes() bytes.
 */
int qsx_rk4_proj_block_build(const void* D, int m, int64_t batch, int K,
                             const double* proj, int nproj, void* out, void* stream);
size_t qsx_rk4_proj_block_workspace_bytes(int m, int64_t batch, int K, int nsteps,
                                          int nproj);
int qsx_rk4_proj_block_mean(const void* matrix, int m, int64_t batch, int K, int nsteps,
                            const double* y0, int64_t y0_stride, int nproj,
                            double* out_mean, void* workspace, size_t workspace_bytes,
                            int32_t* status, void* stream);

/*
 * Hierarchical equations of motion (HEOM).  Replaces HEOMModel.HEOM_tensor
 * and equation_of_motion (qspectra/dynamics/heom.py:228-244, 298-443) by a
 * structured generator on one Liouville block XY (nx x ny, column stacked)
 * per hierarchy node n:
 *   d rho_n/dt = uc { -i (Hx rho_n - rho_n Hy) - shift_n rho_n - W o rho_n
 *                     + sum_t (alpha_t occx_j(a) + beta_t occy_j(b)) rho_{nbr_t} },
 * j = site[n][t].  The host builds the node tables from the ADO enumeration
 * (heom.py:92-174): shift_n = sum_jk n_jk nu_k, up terms (alpha, beta) =
 * (-i m, i m), down terms (-i m c_k, i m conj(c_k)) (heom.py:410-442), W the
 * low-temperature correction times its coefficient (heom.py:386-408), and the
 * transposed tables for the Heisenberg picture (heom.py:236-237).
 */
typedef struct {
  int32_t precision;   /* QSX_FP64, or QSX_FP32 (split-word FP32 state) */
  int32_t nx, ny;      /* block dimensions, nx * ny <= 256 */
  int32_t nnodes;      /* hierarchy nodes */
  int32_t nterms;      /* coupling terms per node (padded with nbr = -1) */
  int32_t n_sites;     /* bath sites (rows of occx / occy) */
  int32_t nsteps;      /* RK4 steps */
  int32_t save_every;  /* output every save_every steps */
  int32_t save_nodes;  /* leading nodes saved per output (1 = physical rho) */
  int32_t variant;     /* 0: the library's choice (the persistent cluster form,
                          one launch for the whole loop, when its shared memory
                          fits and every sample's cluster is resident at once;
                          else one launch per RK4 stage); 1: one launch per RK4
                          stage; 2: the cluster form whenever it fits; 3: one
                          launch per RK4 stage with the node commutators
                          -i (Hx rho_n - rho_n Hy) of a tile of 64 node blocks
                          as one 3xTF32 tcgen05 product against
                          L = I (x) Hx - Hy^T (x) I (FP32 blocks up to 8 x 8;
                          other cases as 1); 4: as 1, but with every coupling
                          term of a node visited by every element (blocks up
                          to 8 x 8 otherwise visit only the terms of the
                          sites their row and column couple to) */
  int64_t batch;       /* disorder samples */
  int64_t H_stride;    /* 0: Hx, Hy shared; else per sample [batch][n][n] */
  const double* Hx;    /* real [nx][nx], rotating frame */
  const double* Hy;    /* real [ny][ny] */
  const double* occx;  /* [n_sites][nx] number-operator diagonals */
  const double* occy;  /* [n_sites][ny] */
  const double* W;     /* [nx * ny] low-temperature weights, or NULL */
  const double* shift; /* [nnodes] */
  const int32_t* nbr;  /* [nnodes][nterms] neighbour node, -1 = none (after the
                          node's terms) */
  const int32_t* site; /* [nnodes][nterms], ascending within each node */
  const double* alpha; /* complex128 [nnodes][nterms] */
  const double* beta;  /* complex128 [nnodes][nterms] */
  double unit_convert;
  double h;            /* RK4 step */
  const double* y0;    /* complex128 [batch][nnodes][nx * ny] */
  int64_t y0_stride;   /* 0 = one initial state for all samples */
  double* out_state;   /* complex128 [batch][nsave][save_nodes * nx * ny] or NULL */
  double* out_mean;    /* complex128 [nsave][save_nodes * nx * ny] or NULL */
  void* workspace;
  size_t workspace_bytes;
  int32_t* status;     /* device int: QSX_ERR_NONFINITE on NaN/Inf */
  const double* gamma; /* complex128 [nnodes][nterms]: aki_temp_corr coefficient of
                          each term (heom.py:438-442), or NULL */
  const double* Wraw;  /* [nx * ny] unscaled double-commutator weights the gamma
                          terms multiply (with occ_j(a) - occ_j(b)), or NULL */
} qsx_heom_args;

int qsx_heom_workspace_bytes(const qsx_heom_args* args, size_t* bytes);
/* out = generator applied to x (FP64), both complex128 [batch][nnodes][nx*ny]. */
int qsx_heom_rhs(const qsx_heom_args* args, const double* x, double* out, void* stream);
/* Fixed-step RK4 loop (stage form), the integrate() loop for HEOM. */
int qsx_heom_rk4(const qsx_heom_args* args, void* stream);
size_t qsx_heom_args_bytes(void);

/*
 * RK4 under applied fields, the time loop of simulate_with_fields /
 * simulate_pump (qspectra/simulate/eom.py:77-227):
 *   dy/dt = L y + sum_p a_p(t) C_p y,
 * a_p(t) = -i E_p(t) (conjugated for '+' transitions) tabulated by the host
 * at every stage time: coef complex [nsteps][3][npulses] for t_n,
 * t_n + h/2 and t_n + h.  L complex [batch][m][m] (L_stride elements per
 * sample, 0 = shared), C complex [npulses][m][m] (the restricted commutator
 * maps of the pulses' dipole operators; C_stride elements per sample, 0 =
 * shared, per-sample maps carry randomly oriented dipoles), all in the working precision
 * (complex64 for QSX_FP32, which keeps a split-word state; complex128 for
 * QSX_FP64).  y0 complex128 [batch][m] (y0_stride 0 = shared); out_state
 * complex128 [batch][nsteps / save_every + 1][m].  m <= 1024 and the
 * generator plus field maps must fit in 227 KB of shared memory.
 */
int qsx_rk4_field_batched(const void* L, int64_t L_stride, const void* C,
                          int64_t C_stride, int npulses,
                          const void* coef, int m, int64_t batch, int nsteps, double h,
                          const double* y0, int64_t y0_stride, int save_every,
                          int precision, double* out_state, int32_t* status,
                          void* stream);

/*
 * ZOFE master equation (qspectra/dynamics/zofe.py:121-229), the time loop of
 * a ZOFEModel, optionally under applied fields (simulate/eom.py:77-105).
 * The state vector is the reference's: rho (n x n, column-major) followed by
 * the auxiliary operators O (npm, n_sites, n, n) in column-major order, i.e.
 * O[pm][s][k][l] at n*n + pm + npm (s + n_sites (k + n l)).  The right-hand
 * side (unit_convert times)
 *   rho' = b rho + sum_s L_s rho S_s^H + rho (i H - a^H) + sum_s S_s rho L_s^H
 *   O'   = Gamma[pm][s] L_s - w[pm][s] O + b O - O b
 * with S_s = sum_pm O[pm][s], a = sum_s L_s^H S_s, b = -i H - a, L_s =
 * diag(Ld[s]) (the system-bath couplings carrying the ZOFE sign: minus the
 * site number operators), plus sum_p a_p(t) [V_p, .] on rho and on every O
 * for pulses, not scaled by unit_convert (a_p tabulated at t_n, t_n + h/2, t_n + h as for
 * qsx_rk4_field_batched).  Fixed-step RK4; FP32 keeps a split-word state.
 * One thread-block cluster per sample splits the pseudomodes over its CTAs
 * (cluster 0 = chosen by the library); n <= 32 and at most 4096 state
 * elements per CTA.
 * hermit (ZOFEModel's rho_hermit / ham_hermit, zofe.py:179-192): with
 * QSX_ZOFE_RHO_HERMIT the last rho term is sum_s S_s rho^H L_s^H (the
 * conjugate transpose of the second), and with both flags the third is
 * rho^H (i H - a^H) as well (the right operator is then b^H, which equals
 * i H - a^H for the symmetric H this entry takes).  Field terms act on rho
 * itself in every form.
 */
#define QSX_ZOFE_RHO_HERMIT 1
#define QSX_ZOFE_HAM_HERMIT 2
typedef struct {
  int32_t precision;     /* QSX_FP64 or QSX_FP32 */
  int32_t n;             /* Hilbert-space states */
  int32_t n_sites;       /* sites (couplings L_s) */
  int32_t npm;           /* pseudomodes */
  int32_t nsteps;        /* RK4 steps */
  int32_t save_every;    /* output every save_every steps */
  int32_t npulses;       /* field terms, 0 = free evolution */
  int32_t nproj;         /* projections of rho saved instead of (or beside) states */
  int32_t mode;          /* 0: RK4 loop; 1: evaluate the right-hand side at y0 once */
  int32_t cluster;       /* CTAs per sample, 0 = library's choice, else 1..8 */
  int64_t batch;         /* samples */
  const double* H;       /* real [n][n] rotating-frame Hamiltonian */
  int64_t H_stride;      /* elements between samples, 0 = shared */
  const double* Ld;      /* real [n_sites][n] diagonals of L_s */
  const double* Gamma;   /* complex128 [npm][n_sites], Omega^2 huang */
  const double* w;       /* complex128 [npm][n_sites], i Omega + gamma */
  const double* V;       /* complex128 [npulses][n][n] row-major dipole operators */
  int64_t V_stride;      /* elements between samples, 0 = shared */
  const double* coef;    /* complex128 [nsteps][3][npulses] (mode 1: [1][3][npulses]) */
  const double* proj;    /* complex128 [nproj][n*n] rows over rho (column-major) */
  double unit_convert;
  double h;              /* RK4 step */
  const double* y0;      /* complex128 [batch][M], M = n^2 + npm n_sites n^2 */
  int64_t y0_stride;     /* elements between samples, 0 = shared */
  double* out_state;     /* complex128 [batch][nsteps/save_every + 1][M] or NULL
                            ([...][n*n], rho only, with save_rho_only);
                            mode 1: [batch][M], the right-hand side */
  double* out_proj;      /* complex128 [batch][nsteps/save_every + 1][nproj] or NULL */
  int32_t* status;       /* device int: QSX_ERR_NONFINITE on NaN/Inf */
  int32_t hermit;        /* 0 or QSX_ZOFE_RHO_HERMIT [| QSX_ZOFE_HAM_HERMIT] */
  int32_t save_rho_only; /* 1: out_state keeps rho only (mode 0) */
} qsx_zofe_args;

size_t qsx_zofe_args_bytes(void);
int qsx_zofe_rk4(const qsx_zofe_args* args, void* stream);

/*
 * Batched FP64 symmetric eigensolver for n up to 2048 (the two-exciton
 * block; the reference calls scipy.linalg.eigh per sample,
 * qspectra/hamiltonian.py:310-328): Householder tridiagonalisation (one CTA
 * per matrix), bisection on Sturm counts and inverse iteration (one thread
 * per eigenvalue), back-transform by the reflectors.  H float64 [batch][n][n] symmetric;
 * E float64 [batch][n] ascending; U float64 [batch][n][n], column k the
 * eigenvector of E[k].  Workspace: qsx_eigh_large_workspace_bytes.
 * status: QSX_ERR_NONFINITE when an eigenvalue comes out non-finite.
 */
size_t qsx_eigh_large_workspace_bytes(int n, int64_t batch);
int qsx_eigh_large_batched(const double* H, int n, int64_t batch, double* E,
                           double* U, void* workspace, size_t workspace_bytes,
                           int32_t* status, void* stream);

/*
 * Adjoint of the ensemble-mean projected RK4 loop (no reference
 * counterpart: the reference has no gradients; this differentiates the
 * linear_response / absorption_spectra path, qspectra/simulate/
 * response.py:15-154, averaged over the ensemble, decorators.py:40-64).
 * Forward: y_{k+1} = (I + D_s) y_k, x_n = scale * sum_s c^T y_{s,n}.
 * Given cotangents g[n] (complex128 [nsteps+1], PyTorch's convention for
 * complex tensors), writes gradD complex128 [batch][m][m] =
 * sum_k lam_{k+1} y_k^H with lam_N = scale g_N conj(c) and
 * lam_k = (I + D)^H lam_{k+1} + scale g_k conj(c), and, when grady0 is not
 * NULL, lam_0 per sample (complex128 [batch][m]).  checkpoints complex128
 * [batch][nck][m] hold y at steps 0, ck_every, 2 ck_every, ... (nck *
 * ck_every >= nsteps); each segment is recomputed on the device.  m <= 32.
 */
int qsx_rk4_adjoint_batched(const double* D, int m, int64_t batch, int nsteps,
                            const double* checkpoints, int ck_every, int nck,
                            const double* c, const double* g, double scale,
                            double* gradD, double* grady0, void* stream);

/*
 * Two-exciton (f) manifold in operator form, for third_order_response
 * (qspectra/simulate/response.py:267-337) at site counts where the dense
 * 'gef' Redfield tensor (qspectra/dynamics/redfield.py:9-74, n^4 entries)
 * cannot be built.  N sites, P = N(N-1)/2 pair states (k < l, the
 * all_states order of qspectra/operator_tools.py:122-152).
 *
 * qsx_fblock_tensor: the eigenbasis tensor of the f manifold,
 *   Y_i[c][d] = uc * (U^T diag(occ_i) U)[c][d] * C(E_d - E_c)
 * (the per-manifold restriction of redfield.py:41-69), so that
 * M_i^f = U Y_i U^T.  E float64 [batch][P] and U float64 [batch][P][P]
 * (columns = eigenvectors) of the f-block Hamiltonian; site_pairs int32
 * [N][N-1] lists the pair states containing each site.  Y is written in the
 * working precision (FP32 or FP64) as [batch][P][2N][P]: planes 0..N-1 hold
 * Re Y_i, planes N..2N-1 hold Im Y_i.
 */
int qsx_fblock_tensor(const double* E, const double* U, int P, int N,
                      const int* site_pairs, int64_t batch, double temperature,
                      double reorg_energy, double cutoff_freq, int matsubara_cutoff,
                      int discard_imag_corr, double unit_convert, int precision,
                      void* Y, void* stream);

/*
 * qsx_fe_generator: column operators of the 'fe' Liouville block,
 *   Q[s][q][b][r] = M_b^f[q][r] - G^f[q][r] - i uc H^f[q][r],
 * G^f = sum_i diag(occ_i) M_i^f.  M in the plane layout of
 * qsx_fblock_tensor (after both basis transforms), H float64 [batch][P][P]
 * rotating-frame f-block Hamiltonian, pair_sites int32 [P][2].  Q complex in
 * the working precision, [batch][P][N][P].
 */
int qsx_fe_generator(const void* M, const double* H, int P, int N, int64_t batch,
                     const int* pair_sites, double unit_convert, int precision,
                     void* Q, void* stream);

/*
 * qsx_fe_heisenberg_rk4: fixed-step RK4 of the Heisenberg-picture 'fe' block
 * (the plain transpose of L restricted to 'fe', liouville_space.py:316-341),
 * as integrate() runs it for the t3 leg of the excited-state-absorption
 * pathways (response.py:323-336).  Q from qsx_fe_generator; Ae = G^e + i uc
 * H^e complex [batch][N][N] and Me complex [batch][N][N][N] (Me[i] = M_i^e,
 * site basis, including uc) in the working precision.  y0 complex128
 * [batch][P*N] with stride y0_stride (0 = shared), column-stacked over the
 * block.  out complex128 [batch][nsteps+1][P*N]: the state at every step.
 * FP32 keeps a split-word (hi + lo) state.  Workspace:
 * qsx_fe_heisenberg_workspace_bytes.  status: QSX_ERR_NONFINITE on NaN/Inf.
 */
size_t qsx_fe_heisenberg_workspace_bytes(int P, int N, int64_t batch, int precision);
int qsx_fe_heisenberg_rk4(const void* Q, const void* Ae, const void* Me,
                          const int* pair_sites, int P, int N, int64_t batch,
                          int precision, const double* y0, int64_t y0_stride,
                          int nsteps, double h, double* out, void* workspace,
                          size_t workspace_bytes, int32_t* status, void* stream);

/*
 * qsx_csr_map_batched: out[b][r] = sum_k vals[k] * in[b][cols[k]] over
 * rowptr[r] <= k < rowptr[r+1]: a sparse dipole super-operator
 * (LiouvilleSpaceOperator.commutator, liouville_space.py:151-209) applied to
 * a batch of Liouville vectors.  in complex128 [batch][n_in], out complex128
 * [batch][n_out], vals complex128, rowptr/cols int32.
 */
int qsx_csr_map_batched(const double* in, int64_t n_in, int64_t batch,
                        const int* rowptr, const int* cols, const double* vals,
                        int n_out, double* out, void* stream);

/*
 * Direct discrete Fourier transform of uniformly sampled signals,
 *   X[b][k] = dt * sum_n x[b][n] exp(i * sign * (freqs[k] - rw_freq) * uc * t_n),
 * t_n = t0 + n dt.  With freqs on the FFT grid this equals fourier_transform
 * (qspectra/simulate/utils.py:154-219: zero padding to a symmetric time
 * grid, fftshift/fft/ifftshift, sign flip, + rw_freq); any other grid
 * (e.g. 1024 frequencies in a window) is evaluated directly.
 * x complex128 [batch][nt], freqs float64 [nf] (device), X complex128 [batch][nf].
 */
int qsx_dft_batched(const double* x, int nt, int64_t batch, double t0,
                    double dt, const double* freqs, int nf, double rw_freq,
                    double unit_convert, int sign, double* X, void* stream);

/*
 * The same transform for signals from FP32 propagation (the FP32 contract,
 * 1e-4): phases anchored in FP64 every 128 samples, rotated and summed in
 * FP32 between anchors, slices added in FP64 (relative error of order 1e-6).
 * Same arguments; nt <= 24576.
 */
int qsx_dft_batched_f32(const double* x, int nt, int64_t batch, double t0,
                        double dt, const double* freqs, int nf, double rw_freq,
                        double unit_convert, int sign, double* X, void* stream);

/*
 * Two-dimensional transform of a third-order signal for the 2D spectrum
 * (two_dimensional_spectra, qspectra/simulate/response.py:430-455: the t1
 * transform with sign -1, then the t3 transform, each as
 * fourier_transform, qspectra/simulate/utils.py:154-219), both axes in one
 * launch, FP64:
 *   X[k1][b][k3] = dt1 dt3 sum_{n1, n3} x[n1 s1 + b sb + n3 s3]
 *                  exp(i sign1 (f1[k1] - rw) uc (t01 + n1 dt1))
 *                  exp(i sign3 (f3[k3] - rw) uc (t03 + n3 dt3)),
 * x complex128 with element strides s1, sb, s3 (the engine's (t1, t2, t3)
 * array: s1 = batch n3, sb = n3, s3 = 1); X complex128 [nf1][batch][nf3].
 * n1 <= 1600.
 */
int qsx_dft2_batched(const double* x, int n1, int64_t batch, int n3, int64_t s1,
                     int64_t sb, int64_t s3, double t01, double dt1, const double* f1,
                     int nf1, int sign1, double t03, double dt3, const double* f3,
                     int nf3, int sign3, double rw_freq, double unit_convert, double* X,
                     void* stream);

#ifdef __cplusplus
}
#endif
#endif /* QSX_H_ */
