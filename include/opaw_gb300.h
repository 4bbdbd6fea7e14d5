/*
 * opaw_gb300.h — C ABI of the GB300 (sm_103a) OPAW-TDDFT propagation path.
 *
 * The reference (minhchemucla/OPAW-TDDFT) is Fortran 90 over module globals
 * with no FFI layer.  Each entry point below replaces one reference subroutine
 * (cited beside it) and is callable from Fortran through ISO_C_BINDING: plain
 * pointers, sizes and doubles, an int status return, no C++ or torch types.
 *
 * Conventions shared with the reference:
 *   - grids are (nx,ny,nz), x fastest (Fortran column-major), index
 *     ix + nx*(iy + ny*iz) with 0-based ix,iy,iz;
 *   - complex data is interleaved (re,im) complex128 (Fortran complex*16) on
 *     the host; device buffers are complex128 (OPAW_C128) or complex64
 *     (OPAW_C64);
 *   - ir_start and local_grid are 1-based, as the reference stores them;
 *   - per-atom ms x ms matrices (D_ij, rho_ij) are column-major (i fastest);
 *   - set 0 is the unperturbed orbital set (phi_bar), set 1 the kicked one
 *     (phi_bar_pert).
 *
 * Errors: every function returns OPAW_OK (0) or a nonzero status and never
 * exits the process (the reference calls `stop`).  opaw_last_error() returns
 * the message of the last failure on the calling thread.
 */
#ifndef OPAW_GB300_H
#define OPAW_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum opaw_status {
  OPAW_OK = 0,
  OPAW_ERR_ARG = 1,       /* bad argument (size, index, null pointer) */
  OPAW_ERR_CUDA = 2,      /* CUDA runtime failure */
  OPAW_ERR_STATE = 3,     /* call out of order (e.g. no orbitals uploaded) */
  OPAW_ERR_BOX = 4,       /* projector box outside a non-periodic grid */
  OPAW_ERR_NOMEM = 5,     /* device allocation failed */
  OPAW_ERR_NONFINITE = 6, /* NaN/Inf detected in a checked reduction */
  OPAW_ERR_NODEV = 7      /* no CUDA device */
};

/* element type of a device orbital buffer.  OPAW_C128_DD: complex128 data
 * whose Gram matrices and rotations (opaw_gram_dev, opaw_gram_herm_dev,
 * opaw_rotate_dev) are computed in double-FP32 arithmetic (hi + lo FP32
 * pairs, about 1e-14 relative instead of FP64's 1e-16, several times faster
 * on a GPU whose FP64 rate is 1/64 of FP32); elsewhere it is not accepted */
enum opaw_dtype { OPAW_C128 = 0, OPAW_C64 = 1, OPAW_C128_DD = 2 };

/* arithmetic of a propagation: FP64 everywhere, or FP32 FFT / v_ks /
 * projector work with FP64 RK4 accumulation, D_ij, S^-1/2 coefficients and
 * dipole */
enum opaw_precision { OPAW_PREC_FP64 = 0, OPAW_PREC_MIXED = 1 };

/*
 * System description: the operator tables the reference builds once in its
 * set-up (ncpaw_libpaw_prepare.f90, prepare_paw.f90, g3d.f90, vloc.f90) and
 * keeps in main_mod / atom_mod (4_main.f90:1-51, 3_atom.f90:17-101).
 * Per-atom arrays are concatenated in atom order.
 */
typedef struct opaw_system {
  int nx, ny, nz;          /* grid (main_mod nx,ny,nz) */
  double dx, dy, dz;       /* spacing, Bohr */
  double ekcut;            /* kinetic clamp, Ha (ek.f90:42-44); <=0: none */
  int scale_vh;            /* Hartree box factor: 2 non-periodic (MT), 1 periodic */
  int periodic;            /* 0: Martyna-Tuckerman, 1: periodic 4pi/k^2 */
  double rnel;             /* electron count for the charge renormalisation */
  int natom;
  const int *ir_start;     /* [3*natom] 1-based box origin (get_irs.f90:22-26) */
  const int *nrough;       /* [3*natom] box extents (read_paw.f90:250-253) */
  const int *ms;           /* [natom] projectors per atom */
  const double *p3d;       /* raw projectors p~, per atom [ms][nbox], box x fastest */
  const double *p3d1;      /* orthogonalised projectors p1, same layout */
  const double *s;         /* [sum ms] spectrum s_i of the p1 overlap (transform_p3d.f90:53-55) */
  const double *sinv;      /* [sum ms] used by sn_phi for n = -1 */
  const int *ngrid;        /* [natom] compensation-sphere points (map_localgrid.f90) */
  const int *local_grid;   /* [3*sum ngrid] 1-based ix,iy,iz per point */
  const int *nlm;          /* [natom] (2*nl-1)^2 shape-function channels */
  const double *g3d;       /* per atom [nlm][ngrid], ig fastest (local_g3d) */
  const double *qijlm;     /* per atom [ms][ms][nlm], lm fastest (qijlm) */
  const double *vloc;      /* [nn] local ionic potential (vloc_tot) */
  const double *ncoret;    /* [nn] pseudo core density */
  const double *dij0;      /* per atom [ms*ms] frozen on-site term D0 */
  const double *eijkl;     /* per atom [ms^4] on-site Hartree tensor: D_H_ij = sum_kl E[i,j,k,l] rho_kl */
  double dij_max;          /* |D_ij| clamp (param_dij_max, 0_parameter.f90:17) */
  /* On-site exchange-correlation term of D_ij, D_xc = dE_xc/drho_ij of the
   * one-centre densities (libpaw pawdenpot + pawdij with the first-order
   * moment development pawxcdev = 1, LDA, nspden = 1: m_paw_denpot.F90:136,
   * 2_m_pawxc.F90 pawxcm, 4_m_pawdij.F90 pawdijxcm).  rad_n == NULL leaves
   * the term out.  Per atom, concatenated in atom order: */
  const int *rad_n;        /* [natom] radial mesh points of the PAW sphere (pawrad%mesh_size) */
  const double *rad_r;     /* per atom [rad_n] radii r_k > 0 (pawrad%rad) */
  const double *rad_w;     /* per atom [rad_n] weights: int_0^rpaw f dr = sum_k w_k f(r_k) (simp_gen) */
  const int *nphi;         /* [natom] radial partial waves (pawtab%basis_size) */
  const double *phi;       /* per atom [nphi][rad_n] all-electron u(r) = r phi(r) (pawtab%phi) */
  const double *tphi;      /* per atom [nphi][rad_n] pseudo u~(r) = r phi~(r) (pawtab%tphi) */
  const double *coredens;  /* per atom [rad_n] core density n_c(r) (pawtab%coredens) */
  const double *tcoredens; /* per atom [rad_n] pseudo core density (pawtab%tcoredens) */
  const int *proj_lmn;     /* [3 * sum ms] per projector: l, m (-l..l, real Y_lm of ylm.f90), partial
                            * wave index (pawtab%indlmn) */
} opaw_system;

typedef struct opaw_ctx opaw_ctx;

/* ---- lifetime ---------------------------------------------------------- */

/* Builds the device copy of every operator table, the kinetic table
 * (ek.f90:1-51, A15) and the Martyna-Tuckerman kernel (vk_TuMa.f90:2-117,
 * vk_scale.f90:23-48, A14).  Replaces ncpaw_libpaw_prepare's device-side
 * outputs.  Checks every projector box (get_irs.f90:30-38). */
int opaw_dev_init(const opaw_system *sys, opaw_ctx **out);
int opaw_dev_free(opaw_ctx *ctx);
const char *opaw_last_error(void);
/* the cudaStream_t all work of this context is issued on (non-blocking: a
 * caller that writes a device input on another stream orders that work
 * before the call itself, e.g. by issuing it on this stream) */
void *opaw_stream(opaw_ctx *ctx);
/* number of this library's kernels launched since the context was made */
int64_t opaw_kernel_launches(opaw_ctx *ctx);
/* live timing of the mixed step's dominant kernel (the fused RK4 / S^-1/2 /
 * density pass over the grid points outside the projector boxes): between
 * begin and end every launch of it is bracketed by CUDA events on the
 * context's stream, and its algorithmic bytes (each array element it must
 * read or write, once) are added up.  end waits for the stream and returns
 * the summed device time, the launches and the bytes.  Measurement plumbing
 * with no counterpart in the reference. */
int opaw_ktime_begin(opaw_ctx *ctx);
int opaw_ktime_end(opaw_ctx *ctx, double *ms, int *launches, double *bytes);

/* Launch-shape autotuner (no reference counterpart).  Some launch shapes
 * have candidates that compute bit-identical results with different speed
 * (L2 prefetch distance of the copy plane pass, lines per CTA of the z pass,
 * orbitals per CTA of the box terms, block size of the dense stage pass);
 * the context times each candidate twice on the launches it makes anyway and
 * keeps the fastest per launch shape.  mode 1 (the default): timing;
 * 2: frozen, the sites decided so far keep their choice, the others take
 * their default and nothing more is timed (for a timed region); 0: off, every
 * site takes its default. */
int opaw_tune_enable(opaw_ctx *ctx, int mode);
/* the tuner's state as JSON, [{"site", "candidates", "ms", "chosen"}, ...]
 * (chosen -1: still timing); writes at most len bytes with the terminating
 * NUL, *needed = the full length + 1 */
int opaw_tune_report(opaw_ctx *ctx, char *buf, int64_t len, int64_t *needed);

/* waits for all work issued on the context's stream (the *_dev entry points
 * below are asynchronous on that stream) */
int opaw_sync(opaw_ctx *ctx);

/* ---- orbital storage (psi stays resident between calls) ------------------ */

/* Copies norb complex128 orbitals (nn each) of `set` host->device.
 * Replaces the scatter of phi_bar_tot (tddft.f90:246-267). */
int opaw_psi_upload(opaw_ctx *ctx, int set, const double *psi, int norb);
int opaw_psi_download(opaw_ctx *ctx, int set, double *psi, int norb);
/* device pointer of the resident complex128 orbitals of `set` */
void *opaw_psi_device(opaw_ctx *ctx, int set);

/* ---- operator state (per set) ------------------------------------------- */

int opaw_set_vks(opaw_ctx *ctx, int set, const double *vks);   /* [nn] */
int opaw_get_vks(opaw_ctx *ctx, int set, double *vks);
int opaw_set_dij(opaw_ctx *ctx, int set, const double *dij);   /* [sum ms^2] */
int opaw_get_dij(opaw_ctx *ctx, int set, double *dij);
int opaw_get_rhoij(opaw_ctx *ctx, int set, double *rhoij);     /* [sum ms^2] */
int opaw_get_density(opaw_ctx *ctx, int set, double *dens);    /* [nn] dens / dens_pert */
int opaw_get_nhat(opaw_ctx *ctx, int set, double *nhat);       /* [nn] */

/* ---- per-routine operators over device buffers -------------------------
 * pin/out are device pointers to norb orbitals of nn points, dtype elements;
 * `set` selects v_ks / D_ij (unpert or pert twin). */

/* h_phi / h_phi_pert (hphi.f90:1-66, hphi_pert.f90:1-62) */
int opaw_h_apply_dev(opaw_ctx *ctx, int set, int dtype, const void *pin, void *hp, int norb);
/* sn_phi (snphi.f90:1-49): n in {-1, -0.5, 0.5, 1}; n == -1 uses sinv */
int opaw_sn_apply_dev(opaw_ctx *ctx, int dtype, double n, const void *pin, void *sp, int norb);
/* shs / shs_pert (shs.f90:3-23,50-70) */
int opaw_shs_apply_dev(opaw_ctx *ctx, int set, int dtype, const void *pin, void *pout, int norb);
/* proj / proj1 (proj.f90:1-44, proj1.f90:1-46): ca[orb][atom offset + i],
 * complex128 host output, which = 0 raw p~, 1 orthogonalised p1 */
int opaw_proj_dev(opaw_ctx *ctx, int which, int dtype, const void *pin, int norb, double *ca);

/* Teter-Payne-Allan kinetic preconditioner of the ground-state eigensolver
 * (no reference counterpart: the reference's Chebyshev-filtered SCF,
 * chebyr_m.f90, uses none): out_b = F^-1 [K(|k|^2/2 / ekin[b]) F pin_b] with
 * K(x) = (27+18x+12x^2+8x^3)/(27+18x+12x^2+8x^3+16x^4), ekin a host array of
 * norb positive kinetic energies; asynchronous on the context's stream
 * (the host array is consumed before the call returns); out may equal pin */
int opaw_precond_kinetic_dev(opaw_ctx *ctx, int dtype, const void *pin, const double *ekin, void *out, int norb);
/* kinetic energies ekin[b] = <x_b|T|x_b> / <x_b|x_b> of norb device
 * orbitals, T the kinetic operator of the Hamiltonian (ek.f90:1-51: |k|^2/2
 * capped at ekcut); the preconditioners' energy scale; host output, waits
 * for the stream */
int opaw_kinetic_energy_dev(opaw_ctx *ctx, int dtype, const void *x, int norb, double *ekin);

/* ---- learned preconditioner (no reference counterpart: the reference's
 * ground state comes from a Chebyshev-filtered SCF without preconditioning,
 * chebyr_m.f90:1-48).  A 3-layer 3D convolutional network (3^3 kernels, 16
 * channels, BF16 weights and activations, FP32 accumulation on the tensor
 * cores) maps the normalised residual r / |r| of an orbital and v_ks - eps
 * to a correction added to the Teter-Payne-Allan preconditioner's output.
 * Parameters: 3 layers of [27 taps][16 ci][16 co] weights then 16 biases
 * (float, 3 * 6928 values); activation channels are stored as 16 BF16
 * values per voxel ([batch][z][y][x][16], unused channels zero). ---- */
typedef struct opaw_net opaw_net;
int opaw_net_create(unsigned long long seed, opaw_net **out);
int opaw_net_free(opaw_net *net);
int opaw_net_params(opaw_net *net, float *params);
int opaw_net_set_params(opaw_net *net, const float *params);
int64_t opaw_net_launches(opaw_net *net);
/* forward pass of a host batch x (BF16 bits, [batch][nz][ny][nx][16]) into
 * out (float, [batch][nz][ny][nx][16]; channels 0, 1 are the correction) */
int opaw_net_forward(opaw_net *net, int batch, int nz, int ny, int nx, const uint16_t *x, float *out);
/* loss = sum over the interior voxels (margin voxels from each face) of
 * |out - tgt|^2 / count, and its gradient with respect to the parameters
 * (float, params layout), of a host batch of P^3 patches; tgt [batch][P^3][2] */
int opaw_net_loss_grad(opaw_net *net, int batch, int P, int margin, const uint16_t *x, const float *tgt,
                       double *loss, float *grad);
/* training patches from device fields of a context's grid: r, t complex128
 * [norb][nn] (residuals and targets), per orbital eps and scale (host),
 * origins [npatch][4] = (orbital, z0, y0, x0), periodic wrap; stored in the
 * net at patch indices first .. first + npatch - 1 */
int opaw_net_add_patches(opaw_net *net, opaw_ctx *ctx, const void *r, const void *t, int norb, const double *eps,
                         const double *scale, int npatch, const int *origins, int P, int first);
/* nsteps Adam steps (learning rate lr) on minibatches of `batch` of the first
 * npatch stored patches; losses[s] the loss of step s (may be NULL) */
int opaw_net_train(opaw_net *net, int npatch, int P, int margin, int nsteps, int batch, double lr, double *losses);
/* w = K r + |r| N(r / |r|, v_ks - eps) for norb device orbitals of the
 * context (K: opaw_precond_kinetic_dev with ekin); eps, ekin host [norb] */
int opaw_precond_learned_dev(opaw_ctx *ctx, opaw_net *net, int dtype, const void *r, const double *eps,
                             const double *ekin, void *w, int norb);

/* fft3d_forward / fft3d_backward (lib/library_fftw_v3.f90:56-83): in-place
 * unnormalised 3D DFT of norb device arrays, sign -1 forward, +1 backward */
int opaw_fft3d_dev(opaw_ctx *ctx, int dtype, void *data, int norb, int sign);

/* Gram matrix G = dv A^H B of two device orbital batches (the orbital Gram
 * of orthog_phi.f90:76-111 and the subspace matrices of diag.f90:49-97),
 * complex128 host output, column-major G[i + na*j] */
int opaw_gram_dev(opaw_ctx *ctx, int dtype, const void *A, int na, const void *B, int nb, double *G);
/* the same for a result known to be Hermitian (A^H A, or A^H H A with H
 * Hermitian; n x n): only the tiles on and above the diagonal are summed, the
 * others are their conjugate mirror images */
int opaw_gram_herm_dev(opaw_ctx *ctx, int dtype, const void *A, const void *B, int n, double *G);
/* subspace rotation out_j = sum_i A_i M[i + na*j] (orthog_phi.f90:148-156,
 * diag.f90:118); M complex128 host, column-major; out must differ from A */
int opaw_rotate_dev(opaw_ctx *ctx, int dtype, const void *A, int na, const double *M, int nb, void *out);
/* orthog_phi (orthog_phi.f90, h_type = 1): canonical orthogonalisation of the
 * resident orbitals of `set`, Psi <- Psi V diag(l)^-1/2 with G = V diag(l) V^H;
 * eig (may be NULL) receives the Gram eigenvalues l ascending */
int opaw_orthog(opaw_ctx *ctx, int set, double *eig);
/* FP64 orthonormalisation of the resident orbitals of `set` entirely on the
 * device (the re-orthogonalisation of the orbital Gram matrix; orthog_phi.f90
 * does it with a host eigensolve): method 0 Cholesky, Psi <- Psi L^-H with
 * G = L L^H; method 1 Loewdin, Psi <- Psi G^-1/2 by Newton-Schulz iteration,
 * for orbitals close to orthonormal (max |G - I| < 0.5, else OPAW_ERR_ARG).
 * offdiag (may be NULL) receives max |G - I| before the step. */
int opaw_orthonormalize_dev(opaw_ctx *ctx, int set, int method, double *offdiag);
/* host-only complex Hermitian eigensolver (cyclic Jacobi) used by
 * opaw_orthog, replacing EISPACK ch (library_1_matrix_all.f90:351-401):
 * H (n x n complex128, column-major, overwritten), w ascending, V columns */
int opaw_herm_eig(int n, double *H, double *w, double *V);

/* ---- host-buffer twins of the operators (Fortran arrays in and out) ---- */

int opaw_h_phi(opaw_ctx *ctx, int set, int dtype, const double *pin, double *hp, int norb);
int opaw_sn_phi(opaw_ctx *ctx, int dtype, double n, const double *pin, double *sp, int norb);
int opaw_shs(opaw_ctx *ctx, int set, int dtype, const double *pin, double *pout, int norb);

/* ---- rebuild chain on the resident orbitals ----------------------------- */

/* tddft_rhoij_2 (tddft_rhoij.f90:75-115) on the resident orbitals of `set`
 * as they are (inside the rebuild the reference calls it on S^-1/2 psi_bar) */
int opaw_rhoij(opaw_ctx *ctx, int set, int precision);
/* tddft_dens_2 (tddft_dens.f90:44-85) on the resident orbitals as they are */
int opaw_density(opaw_ctx *ctx, int set, int precision);
/* get_nhat / get_nhat_pert with the charge renormalisation (nhat.f90:1-43) */
int opaw_nhat(opaw_ctx *ctx, int set);
/* get_pot_tddft_2 (tddft_pot.f90:110-181): v_ks = v_H[n~+n^] + v_xc[n~+n~c] + v_loc */
int opaw_vks(opaw_ctx *ctx, int set);
/* get_dij / get_dij_pert (get_dij.f90:1-156) */
int opaw_dij(opaw_ctx *ctx, int set);
/* ncpaw_make_hamiltonian_tddft_{unpert,pert} (ncpaw_make_hamiltonian.f90:213-281) */
int opaw_rebuild(opaw_ctx *ctx, int set, int precision);

/* vh_sub (vh_big.f90:1-75) on host arrays: vh = Hartree potential of dens */
int opaw_vh(opaw_ctx *ctx, const double *dens, double *vh);
/* rconv (library_vh_convolution_r8_r2c.f90:13-39) on an arbitrary real grid:
 * gout = 1/N ifft(bk * fft(gin)), host arrays of n0*n1*n2 */
int opaw_rconv(int n0, int n1, int n2, const double *gin, const double *bk, double *gout);
/* rconv for callers that cannot allocate device memory (no counterpart in
 * the reference; it exists because some callers of this library cannot call
 * cudaMalloc: a host program that fixed its device memory budget at start-up,
 * or a process whose device allocator belongs to another runtime that a
 * library must not touch).  gin, bk and gout are device arrays of n0*n1*n2
 * doubles owned by the caller; the work runs on `stream` (NULL: the legacy
 * default stream).  The twiddle tables are computed on the device, and the
 * call synchronises `stream` before it returns.  No cudaMalloc, cudaFree or
 * allocating library routine is called: the scratch is a fixed file-scope
 * device array, so
 *   - each extent must be <= 256 with prime factors 2, 3, 5, 7 and
 *     n0*n1*n2 <= 262144 (4 MiB of complex128 scratch, plus 12 KiB of
 *     twiddles, held by every GPU that loads the library until exit);
 *     larger sizes are rejected with OPAW_ERR_ARG;
 *   - the first call on a device (and the first after that device's context
 *     changed) looks up the array's device address (cudaGetSymbolAddress);
 *     make that first call before any stream capture;
 *   - all calls share the one scratch array, which keeps the last call's
 *     contents: calls that overlap on the GPU (different host threads or
 *     streams) race and must not be issued concurrently. */
int opaw_rconv_noalloc(int n0, int n1, int n2, const double *gin, const double *bk, double *gout, void *stream);
/* LDA v_xc (libxc LDA_X + LDA_C_PW, vxc_libxc.f90:15-23), host arrays */
int opaw_vxc_lda(opaw_ctx *ctx, const double *dens, double *vxc, int64_t n);

/* ---- kick, propagation, dipole ------------------------------------------ */

/* excite_psi_bar_pert (tddft_excite.f90:1-16): set 1 = set 0 * exp(-i gamma r_ipol) */
int opaw_excite(opaw_ctx *ctx, int ipol, double gamma);
/* plot_dip (tddft_plot.f90:1-155): dip, dip_pert (3 each) and d_dip = (dip_pert-dip)/gamma */
int opaw_dipole(opaw_ctx *ctx, double gamma, double *dip, double *dip_pert, double *d_dip);
/* excite_psi_bar_pert (tddft_excite.f90:1-16) for nkick kicks at once: kicked
 * set k = set 0 * exp(-i gamma[k] r_{ipol[k]}), k = 0 .. nkick-1.  The kicked
 * sets live in set 1's storage ([kick][orbital][point]; kick 0 is what the
 * set-1 entry points see) and are all propagated against the one unperturbed
 * set: the reference propagates one phi_bar_pert per run (rk4.f90:25-33), and
 * the unkicked propagation does not depend on the kick, so a run per kick
 * repeats the same unperturbed set. */
int opaw_excite_kicks(opaw_ctx *ctx, int nkick, const int *ipol, const double *gamma);
/* copies kicked set `kick` (norb orbitals) to a host array */
int opaw_kick_download(opaw_ctx *ctx, int kick, double *psi, int norb);
/* nsteps iterations of the opaw_tddft loop body (tddft.f90:67-91) for the
 * unperturbed set and every kicked set of opaw_excite_kicks: dip_out
 * [nsteps][3] (the unperturbed dipole), dip_pert_out and d_dip_out
 * [nsteps][nkick][3], d_dip of kick k = (dip'_k - dip) / gamma[k]
 * (tddft_plot.f90:57); any output may be NULL */
int opaw_tddft_steps_kicks(opaw_ctx *ctx, int nsteps, double dt, int precision, double *dip_out,
                           double *dip_pert_out, double *d_dip_out);
/* the mixed-precision form of opaw_tddft_steps_kicks for nctx contexts at
 * once (molecules on their own grids, each with its own kicked sets): after
 * one plain step, two steps of every context are captured once into a CUDA
 * graph with a branch per context and the graph is replayed, so the
 * molecules' kernels overlap and each replay is one launch.  Outputs per
 * context i as for opaw_tddft_steps_kicks (dip_out[i], dip_pert_out[i],
 * d_dip_out[i]; any of the arrays or entries may be NULL).  The reference
 * runs one molecule and one kick per job (tddft.f90:1-95). */
int opaw_ensemble_steps(opaw_ctx *const *ctx, int nctx, int nsteps, double dt, double *const *dip_out,
                        double *const *dip_pert_out, double *const *d_dip_out);
/* nsteps iterations of the opaw_tddft loop body (tddft.f90:67-91):
 * rebuild both sets, rk4_prop_shs (rk4.f90:1-103), plot_dip.  d_dip_out
 * receives 3*nsteps values (may be NULL).  In mixed precision a call of 8 or
 * more steps replays a captured two-step CUDA graph (the launches of
 * opaw_ensemble_steps for one context); fewer steps, or kernel timing on
 * (opaw_ktime_begin), issue the launches one by one, with the same results. */
int opaw_tddft_steps(opaw_ctx *ctx, int nsteps, double dt, double gamma, int precision,
                     double *d_dip_out);
/* the same with everything plot_dip writes per step (tddft_plot.f90:101-104):
 * dip, dip_pert and d_dip, 3*nsteps values each (any may be NULL) */
int opaw_tddft_steps_dip(opaw_ctx *ctx, int nsteps, double dt, double gamma, int precision,
                         double *dip_out, double *dip_pert_out, double *d_dip_out);
/* the same, with psi uploaded from and downloaded to host arrays around the
 * steps (the propdt boundary with Fortran-resident phi_bar/phi_bar_pert) */
int opaw_tddft_steps_host(opaw_ctx *ctx, double *psi, double *psi_pert, int norb, int nsteps,
                          double dt, double gamma, int precision, double *d_dip_out);

#ifdef __cplusplus
}
#endif
#endif /* OPAW_GB300_H */
