/*
 * dftbgpu: GB300-native SCC-DFTB hot path (non-periodic Gamma point: SCC cycle, energy, forces).
 *
 * Plain C-ABI (no C++ or torch types) so that the reference's Fortran host can bind it with
 * iso_c_binding, exactly as it binds MAGMA through extlibs/magma.F90:30-60 over
 * extlibs/magmac.c:24-46. All arrays are caller-owned host memory unless a name ends in _dev.
 * Units are atomic (Bohr, Hartree). Matrices are column-major. Every call returns 0 on success or
 * one of the DFTBGPU_ERR_* codes below; dftbgpu_last_error() gives the message.
 *
 * Which reference call each entry point replaces is stated beside it (paths relative to
 * src/dftbp/ of DFTB+ 25.1).
 */
#ifndef DFTBGPU_H
#define DFTBGPU_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
  DFTBGPU_OK = 0,
  DFTBGPU_ERR_ARGS = 1,              /* invalid argument / size */
  DFTBGPU_ERR_CUDA = 2,              /* CUDA runtime error */
  DFTBGPU_ERR_NOT_POSDEF = 3,        /* overlap matrix not positive definite (cf. eigensolver.F90:1232) */
  DFTBGPU_ERR_SCC_NOT_CONVERGED = 4, /* SCC not converged and convergent_only set (main.F90:1679-1690) */
  DFTBGPU_ERR_FERMI = 5,             /* Fermi level search failed (dftb/etemp.F90:179) */
  DFTBGPU_ERR_ITER_CAP = 6,          /* a bounded device iteration hit its cap (eigensolver) */
  DFTBGPU_ERR_STATE = 7,             /* call order violated (e.g. forces before scc) */
  DFTBGPU_ERR_NO_DEVICE = 8
};

/* Precision forms of the SCC cycle. */
enum {
  DFTBGPU_PREC_FP64 = 0,   /* plain FP64 drop-in */
  DFTBGPU_PREC_MIXED = 1   /* FP32 eigensolves (transform, tridiagonalisation, divide and conquer,
                              back-transformation, density matrix) for the early SCC iterations;
                              then one FP64 eigensolve with all eigenvectors, first-order
                              density-matrix perturbation updates around it (FP32 GEMMs on the
                              potential change), and FP64 again at the perturbatively converged
                              charges. Cholesky, Fermi filling, Mulliken, energies and mixing stay
                              FP64; the cycle only ends on a converged FP64 iteration */
};
/* Iteration kind recorded by dftbgpu_scc_history besides the two precision values above. */
enum { DFTBGPU_ITER_PERTURB = 2 };

typedef struct dftbgpu_ctx dftbgpu_ctx;

/* SCC options; field meaning as in the HSD input the reference parses (dftbplus/parser.F90). */
typedef struct {
  double kT;              /* Filling = Fermi { Temperature } (Ha) */
  double scc_tol;         /* SCCTolerance: max |q_out - q_in| per mixed charge (e) */
  int max_iter;           /* MaxSCCIterations */
  int min_iter;           /* MinSCCIterations (default 1) */
  double mix_alpha;       /* Broyden MixingParameter (0.2) */
  double mix_omega0;      /* InverseJacobiWeight (0.01) */
  double mix_min_weight;  /* MinimalWeight (1.0) */
  double mix_max_weight;  /* MaximalWeight (1e5) */
  double mix_weight_fac;  /* WeightFactor (1e-2) */
  double net_charge;      /* Charge (e); N_el = sum(reference occupations) - net_charge */
  int precision;          /* DFTBGPU_PREC_* */
  int convergent_only;    /* ConvergentSCCOnly: return DFTBGPU_ERR_SCC_NOT_CONVERGED if 1 */
  double mixed_switch_tol;/* mixed form: leave the FP32 eigensolves once max|q_out - q_in| < this
                             (0 = default: 3e-3 single system, 1e-3 batched); the converged
                             iteration is always FP64 */
} dftbgpu_scc_opts;

/* Energy terms as in dftb/energytypes.F90 (TEnergies) for this path. */
typedef struct {
  double EnonSCC, Escc, Erep, Eband, TS, E0, Etotal, EMermin;
} dftbgpu_energies;

/* Fill opts with the reference's defaults (parser.F90:5786-5790, Fermi kT = 0). */
void dftbgpu_default_opts(dftbgpu_scc_opts *opts);

/* Context lifecycle: one GPU, one stream per context. Replaces the MAGMA bring-up
 * extlibs/magmac.c:24-46 (dftbp_extlibs_magma_get_gpus_available) / common/gpuenv.F90. */
int dftbgpu_create(dftbgpu_ctx **ctx, int device);
int dftbgpu_destroy(dftbgpu_ctx *ctx);
const char *dftbgpu_last_error(const dftbgpu_ctx *ctx);

/*
 * Species data and Slater-Koster tables, uploaded once. Replaces the device-side use of the
 * containers built by readSKFiles (dftbplus/parser.F90:3668-3886) + getFullTable (:4061-4130).
 *   n_shell[nsp], ang_shell[4*nsp] (row-major [sp][shell]), onsite[4*nsp], ref_occ[4*nsp],
 *   hubbu[nsp] (one U per species: non-orbital-resolved SCC).
 *   Ordered pair p = sp1*nsp + sp2: sk_dist[p] grid spacing, sk_rows[p] rows (row j <-> r=(j+1)*dist),
 *   sk_nint[p] integrals; sk_ham/sk_over concatenated over p, each pair column-major (rows fastest).
 *   rep_nspline[p]; rep_data concatenated over p, each [cutoff, a1, a2, a3, x_start[nS],
 *   cubic coeffs 4*(nS-1), last coeffs 6] (dftb/repulsive/splinerep.F90).
 */
int dftbgpu_set_model(dftbgpu_ctx *ctx, int nsp, const int *n_shell, const int *ang_shell,
                      const double *onsite, const double *hubbu, const double *ref_occ,
                      const double *sk_dist, const int *sk_rows, const int *sk_nint,
                      const double *sk_ham, const double *sk_over,
                      const int *rep_nspline, const double *rep_data);

/*
 * Geometry: coords[3*nAtom] (x,y,z per atom, Bohr), species[nAtom] (0-based). The GPU builds the
 * cluster half neighbour list itself (same pairs as dftb/periodic.F90:380-700 for a non-periodic
 * system), then H0 and S (buildH0/buildS, dftb/nonscc.F90:66-181) and the Cholesky factor of S.
 * Replaces the H0/S part of processGeometry (dftbplus/main.F90:1219-1222).
 */
int dftbgpu_set_geometry(dftbgpu_ctx *ctx, int natom, const double *coords, const int *species);
/* Same with device pointers (coords_dev[3*natom], species_dev[natom]); species must also be given
 * on the host (species_host) because the orbital layout is host metadata. */
int dftbgpu_set_geometry_dev(dftbgpu_ctx *ctx, int natom, const double *coords_dev,
                             const int *species_host);
/* Same with the host's neighbour list instead of the one the GPU builds from the coordinates (the
 * cluster case of updateNeighbourListAndSpecies / getNrOfNeighboursForAll, dftb/periodic.F90:380-445
 * and :996-1022): nneigh[natom] the neighbours of each atom within the SK cutoff (nNeighbourSK),
 * ineigh[(maxneigh + 1) * natom] their indices laid out as iNeighbour(0:maxNeighbour, nAtom) (entry 0
 * the atom itself), 0-based. Each pair counts once, whichever atom lists it; an index outside
 * 0..natom-1 (a periodic image) is rejected with DFTBGPU_ERR_ARGS. Pairs beyond the SK cutoff
 * contribute nothing; pairs within it that the list leaves out are left out of H0 and S. */
int dftbgpu_set_geometry_neighbours(dftbgpu_ctx *ctx, int natom, const double *coords, const int *species,
                                    const int *nneigh, const int *ineigh, int maxneigh);

/*
 * SCC cycle to convergence: potentials, H = H0 + 1/2 S(V+V), generalized eigensolve, Fermi filling,
 * density matrix, Mulliken, energies, Broyden mixing (dftbplus/main.F90:1429-1563 with
 * hamiltonian.F90:148-450, eigenvects.F90:57-102, etemp.F90:59-191, densitymatrix.F90:530-591,
 * populations.F90:120-191, getenergies.F90:47-384, mixer/broydenmixer.F90:180-342).
 *   q_init[natom]: initial atomic populations or NULL for the neutral reference (q0).
 *   Outputs (each may be NULL): energies, ef, eigen[nOrb], filling[nOrb] (x2 spin), q_out[natom]
 *   (Mulliken populations per atom), n_iter, converged.
 */
int dftbgpu_scc(dftbgpu_ctx *ctx, const dftbgpu_scc_opts *opts, const double *q_init,
                dftbgpu_energies *energies, double *ef, double *eigen, double *filling,
                double *q_out, int *n_iter, int *converged);

/*
 * Per-iteration record of the last dftbgpu_scc call, the data of the SCC iteration table the
 * reference prints (dftbplus/mainio.F90:4781-4845, printSccHeader/printSccInfo: iSCC, total
 * electronic energy, its change, SCC error): energy[i] = Eelec = EnonSCC + Escc of iteration i
 * (from its output charges), error[i] = max|q_out - q_in|,
 * precision[i] = DFTBGPU_PREC_FP64 (FP64 eigensolve), DFTBGPU_PREC_MIXED (FP32 eigensolve) or
 * DFTBGPU_ITER_PERTURB (perturbative update around the last FP64 iteration), ms[i] = host wall
 * time of the iteration. Writes min(cap, count) entries (each array may be NULL) and returns the
 * iteration count, or -1 for a NULL context or cap < 0.
 */
int dftbgpu_scc_history(const dftbgpu_ctx *ctx, int cap, double *energy, double *error, int *precision,
                        double *ms);

/*
 * Batched form: many independent molecules (ragged sizes, at most 768 orbitals and 1024 atoms each)
 * sharing the context's model, solved together. The reference has no batched entry point: its
 * counterpart is one dftbgpu_set_geometry + dftbgpu_scc (+ dftbgpu_gradients) per molecule, i.e.
 * one processGeometry call per system (dftbplus/main.F90:1088-1863). Each SCC iteration advances
 * every unconverged molecule by one iteration (one CTA per molecule, the iteration captured as a
 * CUDA graph); molecules stop individually once converged.
 *   set_geometries: atom_off[nmol+1] (atom_off[0] = 0), coords[3*natom] (x,y,z per atom, Bohr,
 *     molecules concatenated), species[natom] (0-based). DFTBGPU_ERR_NOT_POSDEF names the first
 *     molecule whose overlap is not positive definite.
 *   scc: opts as for dftbgpu_scc (net_charge applies to each molecule; DFTBGPU_PREC_MIXED runs FP32
 *     eigensolves per molecule until its SCC error drops below mixed_switch_tol, then FP64).
 *     Outputs (each may be NULL): energies[nmol], q_out[natom] (Mulliken populations), n_iter[nmol],
 *     converged[nmol]. With convergent_only, DFTBGPU_ERR_SCC_NOT_CONVERGED names the first
 *     unconverged molecule (outputs are still written).
 *   gradients: grad[3*natom] of the last batched SCC (energy gradients, as dftbgpu_gradients).
 */
int dftbgpu_batch_set_geometries(dftbgpu_ctx *ctx, int nmol, const int *atom_off, const double *coords,
                                 const int *species);
/* Same with the coordinates already on the device (coords_dev[3*natom]); atom_off and species on
 * the host (the orbital layout is host metadata). */
int dftbgpu_batch_set_geometries_dev(dftbgpu_ctx *ctx, int nmol, const int *atom_off, const double *coords_dev,
                                     const int *species);
int dftbgpu_batch_scc(dftbgpu_ctx *ctx, const dftbgpu_scc_opts *opts, dftbgpu_energies *energies,
                      double *q_out, int *n_iter, int *converged);
int dftbgpu_batch_gradients(dftbgpu_ctx *ctx, double *grad);

/*
 * Energy gradient (not forces) of the converged state, grad[3*natom] (x,y,z per atom).
 * Energy-weighted density matrix + derivative_blockEuclidean (dftb/forces.F90:548-669, FD SK
 * derivatives nonscc.F90:428-484) + SCC double-counting (scc.F90:794-843) + repulsive
 * (repulsive/twobodyrep.F90:273-332). Replaces main.F90:1777-1800.
 */
int dftbgpu_gradients(dftbgpu_ctx *ctx, double *grad);
int dftbgpu_gradients_dev(dftbgpu_ctx *ctx, double *grad_dev);

/*
 * Gradients of the converged Mermin free energy with respect to the model parameters (the
 * differentiable form; the reference has no counterpart, its closest relatives being the force
 * contraction forces.F90:548-669 and the SK interpolation slakoeqgrid.F90:183-244 it differentiates):
 *   dE_dskham, dE_dskover: same layout and length as sk_ham / sk_over of dftbgpu_set_model (one
 *     value per grid point, integral and ordered species pair); dE_dhubbu[nsp].
 * Uses the variational property of the SCC energy (explicit derivatives at fixed rho, W and charges).
 * Each output may be NULL. Accumulation uses atomics: results are reproducible to rounding only.
 */
int dftbgpu_grad_params(dftbgpu_ctx *ctx, double *dE_dskham, double *dE_dskover, double *dE_dhubbu);

/* Sizes and per-orbital Mulliken populations of the converged state (qOutput, mOrb x nAtom
 * collapsed to the nOrb orbitals in atom order). */
int dftbgpu_n_orbitals(const dftbgpu_ctx *ctx, int *n_orb);
int dftbgpu_get_orbital_populations(dftbgpu_ctx *ctx, double *q_orb);

/*
 * Dense generalized symmetric-definite eigensolver on the GPU: A x = lambda B x, all pairs,
 * eigenvalues ascending. Replaces hegvd / magmaHegvd (math/eigensolver.F90:561-660, :1143-1245):
 * A is overwritten by the eigenvectors (B-orthonormal columns), B by its Cholesky factor (lower).
 * n x n column-major host arrays.
 */
int dftbgpu_sygvd(dftbgpu_ctx *ctx, int n, double *a, double *b, double *w);

/* Debug/inspection of device state for tests: which = 0 H0, 1 S, 2 rho (density matrix),
 * 3 H (last SCC Hamiltonian), 4 W (energy-weighted DM; valid after gradients). out[nOrb*nOrb]. */
int dftbgpu_get_matrix(dftbgpu_ctx *ctx, int which, double *out);

/* Number of this library's kernel launches since creation (for launch accounting). */
long long dftbgpu_kernel_launches(const dftbgpu_ctx *ctx);

/*
 * Phase timers measured with CUDA events on the context's stream (the GPU counterpart of the
 * reference's timer tree, common/environment.F90:97-133). Phases, in order:
 *   0 H0/S build + Cholesky, 1 potentials + H assembly, 2 L^-1 H L^-T, 3 tridiagonalisation,
 *   4 tridiagonal divide and conquer, 5 Fermi filling, 6 back-transformation (Q Z, L^-T Y),
 *   7 density matrix, 8 Mulliken + energies, 9 Broyden mixing, 10 gradients, 11 density-matrix
 *   perturbation (mixed form: reference set-up and perturbative updates), 12 FP64 GEMM (all FP64
 *   GEMM launches, overlapping the phases above), 13 FP32 GEMM (mixed form, likewise), 14 FP64
 *   GEMM as tensor-core digit-slice products (mixed form, likewise; FLOPs counted as the FP64
 *   product's 2mnk, the tensor cores execute 36 BF16 products of it). Single kernels, timed launch
 *   by launch (overlapping the phases above; "flops" holds the work in the unit given): 15 one-stage
 *   tridiagonalisation panel kernel in FP64 (FLOPs of its symmetric matrix-vector products, 2 m^2
 *   per column of trailing order m), 16 two-stage panel QR (bytes: the panel read and written
 *   once), 17 bulge chasing (Householder tasks), 18 two-stage back-transformation of the band stage
 *   (FLOPs 2 n^2 k), 19 one-stage tridiagonalisation panel kernel in FP32 (FLOPs as 15).
 * enable: 1 resets and starts accumulating, 0 stops. read: ms[20], flops[20] (algorithmic FLOPs
 * per phase as counted for the roofline), calls[20]; returns the number of phases written.
 */
int dftbgpu_profile_enable(dftbgpu_ctx *ctx, int enable);
int dftbgpu_profile_read(dftbgpu_ctx *ctx, int nphase, double *ms, double *flops, long long *calls);

/*
 * Allocation-free tridiagonal divide and conquer. This entry point has no counterpart in the
 * reference. It serves callers that cannot call cudaMalloc: a host program whose device memory is
 * all held by another allocator or memory pool (an extra cudaMalloc would fail or fragment it), and
 * a time-stepping loop that must not let an allocation synchronise the whole device between steps.
 * It needs no context and allocates nothing.
 *   n in 1..256 (larger n returns DFTBGPU_ERR_ARGS and does nothing);
 *   d[n] (device): diagonal in, eigenvalues ascending out; e[n-1] (device): off-diagonal, read only;
 *   q[n*n] (device, column-major): eigenvectors out; stream: cudaStream_t or NULL (legacy default).
 * The caller passes inputs and outputs; all scratch is one file-scope device array of about 2.2 MB
 * that every GPU loading the library keeps until process exit. The first call on a device looks
 * up that array's device address with cudaGetSymbolAddress; make that first call before any stream
 * capture. Calls share the array and it keeps the last call's contents (each call clears what must
 * start at zero), so calls that overlap on the GPU (other streams or threads) race and must be
 * serialised by the caller. The call waits for its stream before returning (it reads its status
 * word back). Returns 0, DFTBGPU_ERR_ARGS, DFTBGPU_ERR_ITER_CAP or DFTBGPU_ERR_CUDA.
 */
int dftbgpu_stedc_noalloc(int n, double *d, const double *e, double *q, void *stream);

/*
 * Tensor cores for the perturbative updates of the mixed form (no reference counterpart): when
 * enabled (the default), their FP32 products with m, n >= 128 run as split-BF16 compensated products
 * on the tcgen05 tensor cores (three BF16 pieces per operand, six products, FP32 accumulation,
 * relative error ~2^-22) instead of FP32 FMA. Process-wide; returns the previous setting.
 * dftbgpu_test_gemm_tc runs one such product on host arrays (column-major, flags as the library's
 * triangular GEMM hints) for testing.
 */
int dftbgpu_set_tensor_cores(int enable);
int dftbgpu_test_gemm_tc(dftbgpu_ctx *ctx, char ta, char tb, int m, int n, int k, float alpha, const float *a,
                         int lda, const float *b, int ldb, float beta, float *c, int ldc, int flags);
/*
 * FP64-class products of the mixed form on the tensor cores (no reference counterpart): when
 * enabled (the default), the FP64 GEMMs of the mixed form's FP64 iterations (reduced transform,
 * tridiagonalisation updates, divide-and-conquer merges, back-transformation, density and
 * energy-weighted density matrices) run as exact products of BF16 digit slices on the tcgen05
 * tensor cores: eight signed 7-bit digits per element at a power-of-two scale per row (column),
 * group sums exact in FP32 per 64-wide K block, int64 accumulation. The error of an element is below
 * K max|A_ik| max|B_kj| (2^-53 + K 2^-65), FP64-class. The plain FP64 form always uses FP64
 * arithmetic. Process-wide; returns the previous setting. dftbgpu_test_dgemm_tc runs one such
 * product on host arrays (column-major, flags as the library's triangular GEMM hints).
 */
int dftbgpu_set_fp64_emulation(int enable);
/*
 * FP32-class products of the mixed form on the tensor cores (no reference counterpart): when enabled
 * (the default), the FP32 GEMMs of its FP32 eigensolves (reduced transform, divide-and-conquer
 * merges, back-transformation, density matrix) and of the FP64 iterations' FP32 reference products
 * with m, n, k >= 512 run as exact products of BF16 digit slices on tcgen05: three signed 8-bit digits
 * per element at a power-of-two scale per row (column), six products, group sums exact in FP32 per
 * 64-wide K block, int64 accumulation. The error of an element is below about
 * K max|A_ik| max|B_kj| 2^-23 (FP32-class), with no rounding bias over long K. The plain FP64 form
 * never uses it. Process-wide; returns the previous setting. dftbgpu_test_sgemm_digits runs one such
 * product on host arrays (column-major, flags as the library's triangular GEMM hints).
 */
int dftbgpu_set_fp32_emulation(int enable);
int dftbgpu_test_sgemm_digits(dftbgpu_ctx *ctx, char ta, char tb, int m, int n, int k, float alpha,
                              const float *a, int lda, const float *b, int ldb, float beta, float *c, int ldc,
                              int flags);
/*
 * Kernel of those FP64-class products (no reference counterpart): 0 (the default) runs the
 * single-stage kernel (one 64-wide K block, 128-byte-swizzled, per round of copies, products and
 * readback); 1 feeds the tensor cores through a two-stage pipeline of TMA loads (K-sub-blocks of 32,
 * 64-byte swizzle) and reads the group sums back from tensor memory once per 256-wide K window (it
 * measures slower on GB300). Both give the same FP64-class error bound. Process-wide; returns the
 * previous mode, or -1 for an invalid mode.
 */
int dftbgpu_set_digit_gemm_kernel(int mode);
/*
 * Two-stage reduction for the FP32 eigensolves of the mixed form (no reference counterpart; the
 * reference reaches two-stage reductions through ELPA, elecsolvers/elecsolvertypes.F90:27, and
 * MAGMA's dsygvd_m, math/eigensolver.F90:1143-1245): the matrix is reduced to a band of width 32 with
 * GEMM-based panel updates, the band is chased to tridiagonal form in one persistent kernel, and the
 * eigenvectors are back-transformed through both stages. mode 0: always the one-stage panel
 * tridiagonalisation; 1: always two-stage; 2 (the default): two-stage from 12,000 orbitals on.
 * Process-wide; returns the previous mode, or -1 for an invalid mode (nothing changes).
 */
int dftbgpu_set_two_stage(int mode);
/*
 * Panel kernel of the one-stage tridiagonalisation (no reference counterpart; the reference calls
 * LAPACK dsytrd/MAGMA through math/eigensolver.F90): mode 1 (the default) keeps the trailing
 * matrix of each 32-column panel in shared memory (tiles loaded once per panel by TMA, the rest
 * streamed) with two grid barriers per column, up to 12,288 orbitals in FP32 and 6,144 in FP64;
 * mode 0 re-reads the trailing matrix from memory for every column (three barriers per column,
 * any size); mode 2 is mode 1 with at most 64 CTAs and 8 tile slots (for tests of the streaming
 * path at small sizes). Process-wide; returns the previous mode, or -1 for an invalid mode.
 */
int dftbgpu_set_panel_mode(int mode);
/*
 * Deflation step of the tridiagonal divide and conquer (no reference counterpart; the reference
 * calls LAPACK dstedc/MAGMA): enable = 1 (the default) stages each merge that fits (up to 160 KB of
 * shared memory: 6,144+ entries in FP64, 12,000+ in FP32) on chip, so the sequential deflation scan
 * runs at shared-memory latency and the compaction is a parallel prefix sum; 0 runs every merge in
 * global memory by one thread, as larger merges always do. Same results either way. Process-wide;
 * returns the previous setting.
 */
int dftbgpu_set_dc_staging(int enable);
int dftbgpu_test_dgemm_tc(dftbgpu_ctx *ctx, char ta, char tb, int m, int n, int k, double alpha, const double *a,
                          int lda, const double *b, int ldb, double beta, double *c, int ldc, int flags);
/*
 * Stage-level test hooks (host arrays; used by the parity tests to check each eigensolver stage on
 * its own; they have no counterpart in the reference).
 *   sgemm:   the FP32 FMA product of the mixed form's FP32 iterations (128 x 128 tiles where they
 *            fill the GPU), arguments as dftbgpu_test_gemm_tc.
 *   dgemm:   c = alpha op(a) op(b) + beta c (column-major, lda=m or k as for op 'N'/'T').
 *   tridiag: Householder reduction of the symmetric a (n x n) -> d[n], e[n-1].
 *   stedc:   eigenpairs of the tridiagonal (d, e): d <- eigenvalues ascending, q[n*n] vectors.
 */
int dftbgpu_test_sgemm(dftbgpu_ctx *ctx, char ta, char tb, int m, int n, int k, float alpha, const float *a,
                       int lda, const float *b, int ldb, float beta, float *c, int ldc, int flags);
int dftbgpu_test_dgemm(dftbgpu_ctx *ctx, char ta, char tb, int m, int n, int k, double alpha,
                       const double *a, const double *b, double beta, double *c, int flags);
int dftbgpu_test_tridiag(dftbgpu_ctx *ctx, int n, const double *a, double *d, double *e);
int dftbgpu_test_stedc(dftbgpu_ctx *ctx, int n, double *d, const double *e, double *q);
/*   twostage: two-stage reduction of the symmetric a (n x n) in FP32 (fp32 = 1) or FP64 -> d[n],
 *            e[n-1] and q[n*n] = Q1 Q2 (the accumulated transformation, a = q T q^T). */
int dftbgpu_test_twostage(dftbgpu_ctx *ctx, int n, const double *a, int fp32, double *d, double *e, double *q);
/*   onestage: one-stage reduction (the panel kernel chosen by dftbgpu_set_panel_mode) in FP32 or
 *            FP64 -> d[n], e[n-1] and q[n*n] = Q (a = q T q^T). */
int dftbgpu_test_onestage(dftbgpu_ctx *ctx, int n, const double *a, int fp32, double *d, double *e, double *q);

#ifdef __cplusplus
}
#endif
#endif /* DFTBGPU_H */
