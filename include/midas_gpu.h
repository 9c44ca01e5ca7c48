/*
 * midas_gpu.h -- C ABI of the GB300 (sm_103a) MIDAS VIE-MoM / CBFM hot path.
 *
 * This library replaces the solver layer of nasa-jpl/MIDAS: the subroutines
 * Compute_EFields_MoM (src/Compute_EFields_MoM.f90:1) and
 * Compute_EFields_CBFME / Compute_EFields_CBFME_ACA
 * (src/Compute_EFields_CBFME.f90:1, src/Compute_EFields_CBFME_ACA.f90:1),
 * together with the kernels they call (src/Green_functions.f90,
 * src/Incident_Field.f90, src/Calcul_ACA_matrices.f90,
 * src/getParameters_CBFM.f90) and the MKL ScaLAPACK / PARDISO / GESVD / ZGEMM
 * calls they make.  Each entry point below names the reference interface it
 * stands in for.
 *
 * Conventions (identical to the reference's Fortran arrays):
 *   - complex numbers are interleaved (re, im) doubles, i.e. C `double _Complex`
 *     or Fortran `complex(c_double_complex)`;
 *   - matrices are column-major; the unknown index of cell c and component
 *     p in {x, y, z} is 3c + p (3(c-1)+p, 1-based, in Fortran);
 *   - RHS / field column t is the V polarisation of incident direction t and
 *     column t + ntr its H polarisation (src/Compute_EFields_MoM.f90:557-563);
 *   - angles are in degrees, measured as the reference does: the incident
 *     wave vector is k0 (cos th, sin th cos ph, sin th sin ph)
 *     (src/Incident_Field.f90:32-34);
 *   - index arrays (cell lists, block offsets) use the base given in
 *     midas_gpu_opts.index_base (1 for Fortran callers);
 *   - array arguments may be host or device pointers; the library detects
 *     device memory and then copies nothing;
 *   - every call is synchronous, returns a MIDAS_* status and never aborts
 *     the process (the reference stops with `stop 1` / MPI_ERRORS_ARE_FATAL).
 * One host thread per context; the context owns its CUDA stream.
 */
#ifndef MIDAS_GPU_H
#define MIDAS_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

enum midas_status {
    MIDAS_OK = 0,
    MIDAS_ERR_ARG = 1,            /* invalid argument (size, pointer, option) */
    MIDAS_ERR_CUDA = 2,           /* CUDA runtime / library failure */
    MIDAS_ERR_ALLOC = 3,          /* device allocation failed */
    MIDAS_ERR_SINGULAR = 4,       /* zero pivot ("SINGULAR MATRIX", src/Compute_EFields_MoM.f90:178-181) */
    MIDAS_ERR_NOT_CONVERGED = 5,  /* iterative refinement did not reach ir_tol */
    MIDAS_ERR_STATE = 6,          /* call order: e.g. solve before midas_gpu_set_cells */
    MIDAS_ERR_DEVICE_TIMEOUT = 7, /* a bounded device-side wait expired (kernel returned early) */
    MIDAS_ERR_UNSUPPORTED = 8     /* device is not sm_103 / feature unavailable */
};

/* Dense-solve arithmetic. */
enum midas_solve_mode {
    MIDAS_SOLVE_MIXED = 0,  /* TF32 tensor-core LU (tcgen05) + FP64-residual iterative refinement */
    MIDAS_SOLVE_FP64 = 1    /* plain FP64 LU with partial pivoting (cuSOLVER zgetrf/zgetrs): the baseline */
};

/* Arithmetic of the complex(4)-local fills (Green_s_tr_partial & co). */
enum midas_fill_mode {
    MIDAS_FILL_FAITHFUL = 0, /* reference rounding: FP64 internals rounded to float where the reference rounds */
    MIDAS_FILL_FAST = 1      /* lattice-offset table when the cells lie on one uniform grid */
};

typedef struct midas_gpu_ctx midas_gpu_ctx;

typedef struct {
    int struct_size;   /* sizeof(midas_gpu_opts) */
    int device;        /* CUDA device ordinal (default 0) */
    int index_base;    /* 0 (C) or 1 (Fortran) */
    int solve_mode;    /* enum midas_solve_mode (default MIXED) */
    int fill_mode;     /* enum midas_fill_mode (default FAITHFUL) */
    int ir_max_iter;   /* refinement cap (default 30) */
    double ir_tol;     /* refinement stops when ||b - Z x||_inf <= ir_tol * (||Z||_inf ||x||_inf + ||b||_inf)
                          (default 1e-13) */
    int verbose;       /* 0: silent */
} midas_gpu_opts;

typedef struct {
    int status;             /* same as the return value */
    int ir_iters;           /* refinement steps of the last dense solve */
    double backward_error;  /* final normwise backward error of the last dense solve */
    double anorm;           /* ||Z||_inf (PZLANGE 'I', src/Compute_EFields_MoM.f90:168) */
    int k_total;            /* CBFM: total number of CBFs (K_total, src/Compute_EFields_CBFME.f90:472) */
    int n_far_aca;          /* CBFM+ACA: block pairs represented by ACA factors */
    double t_fill_ms;       /* device time of the fills */
    double t_factor_ms;     /* device time of the factorisations */
    double t_solve_ms;      /* device time of solves + refinement */
    double t_total_ms;      /* wall time of the call */
} midas_gpu_info;

/* Fill *o with the defaults listed above. */
void midas_gpu_default_opts(midas_gpu_opts *o);

/* Create a context on opts->device (NULL opts = defaults).  Replaces the MPI /
 * BLACS set-up of the reference (src/Main_Scattering.f90:226, src/Compute_EFields_MoM.f90:112-123). */
int midas_gpu_init(const midas_gpu_opts *opts, midas_gpu_ctx **ctx);
int midas_gpu_free(midas_gpu_ctx *ctx);
/* Message of the last failure on this context ("" when none). */
const char *midas_gpu_last_error(const midas_gpu_ctx *ctx);

/* Cells of the scatterer for one frequency: centroids, edge Sc, relative
 * permittivity, and k0 = 2 pi / lambda.  Computes a_n, Che = eps - 1, Znnpp and
 * kappa on the device exactly as SetCellsParams (src/SetCellsParams.f90:31-49). */
int midas_gpu_set_cells(midas_gpu_ctx *ctx, int n, const double *xc, const double *yc, const double *zc,
                        const double *sc, const double *eps_re, const double *eps_im, double k0);
/* Read back the per-cell parameters (any output may be NULL); che/znnpp are complex (2n doubles). */
int midas_gpu_get_cell_params(midas_gpu_ctx *ctx, double *a_n, double *che, double *znnpp, double *kappa);

/* Scene preparation on the device.  The reference builds these inputs on the
 * host before the solve; here they are flag passes plus order-preserving
 * compactions, with outputs in the host loops' order.  Output arrays may be
 * host or device memory; index outputs use opts.index_base.
 * midas_gpu_voxelise_sphere: the sphere voxeliser of Discretization
 * (src/Discretization.f90:246-310) for diameter dm and cell edge sc; *ncell
 * receives the count, and up to cap centroids go to xc, yc, zc (NULL = count
 * only). */
int midas_gpu_voxelise_sphere(midas_gpu_ctx *ctx, double dm, double sc, long long cap, double *xc, double *yc,
                              double *zc, long long *ncell);
/* Union of nsph spheres of radius a (centres: 3 doubles each) on one lattice
 * of edge 2a / cells_per_diameter: cells whose centre lies strictly inside a
 * sphere (the reference's inside test), lattice order x slowest (no counterpart
 * in the reference, which reads aggregate shapes from files). */
int midas_gpu_voxelise_spheres(midas_gpu_ctx *ctx, int nsph, const double *centres, double a, int cells_per_diameter,
                               long long cap, double *xc, double *yc, double *zc, long long *ncell, double *edge);
/* Bounding-box split into nx x ny x nz blocks (a partitioner of this library;
 * the reference divides with its own octree, src/Division_blocks.f90): perm
 * (n) lists the cells block by block, stable within a block, and
 * blk_offsets (up to nx ny nz + 1 entries) the non-empty blocks' ranges in the
 * permuted order (the contiguous-by-block ordering of src/Division_blocks.f90:582). */
int midas_gpu_box_partition(midas_gpu_ctx *ctx, int n, const double *xc, const double *yc, const double *zc, int nx,
                            int ny, int nz, int *perm, int *blk_offsets, int *nblocks);
/* Extend_blocks (src/Extend_blocks.f90:46-151) on block-ordered cells: block
 * contours as SetBlockCtrs (src/Division_blocks.f90:1616-1662), neighbours by
 * bounding-sphere distance <= r_b + r_b' + ext_length, and every neighbour cell
 * inside the block's box grown by ext_length + sc / 2.  ext_offsets (nblocks +
 * 1) and up to cap extension cell indices (ext_idx) in the layout
 * midas_gpu_cbfm_solve takes; *ntotal = all extension cells. */
int midas_gpu_extend_blocks(midas_gpu_ctx *ctx, int n, const double *xc, const double *yc, const double *zc,
                            int nblocks, const int *blk_offsets, double ext_length, double sc, int *ext_offsets,
                            long long cap, int *ext_idx, long long *ntotal);

/* Rows [r0, r0+nr) x columns [c0, c0+nc) (0-based unknown indices) of the FP64
 * MoM matrix, column-major nr x nc: compute_Green_s_tr_single_element
 * (src/Compute_EFields_MoM.f90:433-523). */
int midas_gpu_mom_fill(midas_gpu_ctx *ctx, int r0, int nr, int c0, int nc, double *Z);
/* FP64 right-hand sides, 3n x 2ntr: Incident_Field_single_element
 * (src/Compute_EFields_MoM.f90:529-598). */
int midas_gpu_mom_rhs(midas_gpu_ctx *ctx, int ntr, const double *theta, const double *phi, double *V);
/* Incident field with the reference's complex(4) locals on the cells idx[0..ncell)
 * (idx NULL = all cells), 3ncell x 2ntr: Incident_Field (src/Incident_Field.f90:1-63). */
int midas_gpu_incident_field(midas_gpu_ctx *ctx, int ncell, const int *idx, int ntr, const double *theta,
                             const double *phi, double *E);
/* Spherical-wave CBF excitation field with the reference's complex(4) locals on
 * the cells idx[0..ncell) (idx NULL = all cells), 3ncell x 2ntr: sources at
 * 10 block radii from the cells' mean centroid in the directions (theta, phi),
 * Incident_Field_Spherical (src/Incident_Field.f90:65-166). */
int midas_gpu_incident_field_spherical(midas_gpu_ctx *ctx, int ncell, const int *idx, int ntr, const double *theta,
                                       const double *phi, double *E);
/* Block-pair interaction matrix 3n1 x 3n2 (complex(4)-rounded values stored in
 * complex(8)): Green_s_tr_partial (src/Green_functions.f90:96-173). */
int midas_gpu_block_fill(midas_gpu_ctx *ctx, int n1, const int *idx1, int n2, const int *idx2, double *Z);
/* Dense form of the thresholded extended-block matrix handed to PARDISO:
 * SR_Green_s_tr_partial (src/Green_functions.f90:290-562).  Z (3s x 3s) may be
 * NULL; *nnz receives the kept-entry count and *fn (may be NULL) the Frobenius
 * norm of the kept entries (SR_Green_s_tr_partial_FN, :564-806). */
int midas_gpu_sr_fill(midas_gpu_ctx *ctx, int s, const int *idx, double fsr, int homog, double *Z,
                      long long *nnz, double *fn);
/* fSR ladder of setfSR (src/getParameters_CBFM.f90:113-168). */
int midas_gpu_set_fsr(midas_gpu_ctx *ctx, int s, const int *idx, int homog, double res_sr, double *fsr,
                      long long *nnz);
/* Partial-pivot ACA of the unknown block [row0,row0+nrows) x [col0,col0+ncols)
 * (0-based, multiples of 3): Calcul_MatrixZij_ACA (src/Calcul_ACA_matrices.f90:6-219).
 * U is nrows x itmax, V is itmax x ncols (column-major); *rank = nb_iter_out. */
int midas_gpu_aca(midas_gpu_ctx *ctx, int row0, int nrows, int col0, int ncols, double eps, int itmax,
                  double *U, double *V, int *rank);

/* Dense complex solve A X = B (A n x n, B n x nrhs, column-major; B is
 * overwritten by X) with the context's solve_mode.  Stands in for PZGESV
 * (src/Compute_EFields_MoM.f90:173, src/Compute_EFields_CBFME.f90:912). */
int midas_gpu_dense_solve(midas_gpu_ctx *ctx, int n, int nrhs, const double *A, double *B,
                          midas_gpu_info *info);

/* Y = Z X with the MoM matrix Z of compute_Green_s_tr_single_element
 * (src/Compute_EFields_MoM.f90:433-523) applied as an FFT convolution, for cells
 * that lie on one uniform lattice (no counterpart in the reference, which
 * forms Z densely): X and Y are 3n x nrhs column-major complex (host or device).
 * FP64 transforms; returns MIDAS_ERR_UNSUPPORTED when the cells are not on a
 * lattice or a lattice axis spans more than 256 cells. */
int midas_gpu_lattice_matvec(midas_gpu_ctx *ctx, int nrhs, const double *X, double *Y);

/* Krylov solve of the MoM system for cells on one lattice (no counterpart in
 * the reference, whose PZGESV, src/Compute_EFields_MoM.f90:153-198, this
 * complements for systems too large for a dense matrix): GMRES(restart) on the
 * FFT operator of midas_gpu_lattice_matvec, right-hand sides the FP64 incident
 * field of Incident_Field_single_element (src/Compute_EFields_MoM.f90:529-598),
 * all 2ntr columns in lockstep.  E0 (3n x 2ntr, may be NULL = zero) is the
 * initial guess, e.g. a learned predictor's output.  Converged when the TRUE
 * relative residual ||b - Z E|| / ||b|| of every column, recomputed in FP64
 * at each restart, is <= tol.  flags: MIDAS_GMRES_JACOBI right-preconditions
 * with 1 / (1 - Znnpp) per cell.  info->ir_iters = Arnoldi steps taken,
 * info->backward_error = the final true relative residual.  Returns
 * MIDAS_ERR_NOT_CONVERGED after maxit steps (E then holds the last iterate; the
 * dense midas_gpu_mom_solve is the fallback). */
enum midas_gmres_flags { MIDAS_GMRES_JACOBI = 1 };
int midas_gpu_gmres_solve(midas_gpu_ctx *ctx, int ntr, const double *theta, const double *phi, const double *E0,
                          int restart, int maxit, double tol, int flags, double *E, midas_gpu_info *info);

/* Learned initial guess for midas_gpu_gmres_solve (no counterpart in the
 * reference).  A 3-D convolutional network on a grid^3 voxel grid (grid even,
 * <= 128): 16 input channels per voxel -- Re, Im of chi = eps - 1 (0 outside
 * the scatterer) in channels 0-1, Re, Im of the three incident-field components
 * in channels 2-7, Re, Im of chi times each component in 8-13, the mask in 14
 * and 0 in 15 -- and the prediction E = E_inc + mask * net(...), 6 channels
 * (in general: channels 2-7, the base field the network corrects, plus its
 * masked output)
 * (Re, Im of Ex, Ey, Ez).  Four 3x3x3 convolutions (16 -> 32 -> 32 -> 32 -> 6,
 * ReLU), fp16 operands on the
 * tensor cores with FP32 accumulation, FP32 master weights, Adam.  Arrays are
 * voxel-major, x fastest then y then z, one sample after another:
 * inputs [batch][grid^3][16], mask [batch][grid^3] (1 inside, 0 outside), target
 * and E [batch][grid^3][6]; host or device memory.  batch <= 64 and
 * batch * grid^3 <= 2^22.  Parameters are laid out layer by layer, weights
 * [cout][27 taps (dz, dy, dx = -1..1, dx fastest)][cin] then biases [cout], with
 * the last layer's cout padded to 8 (rows 6, 7 stay zero). */
typedef struct midas_gpu_nn midas_gpu_nn;
int midas_gpu_nn_create(midas_gpu_ctx *ctx, int grid, unsigned long long seed, midas_gpu_nn **net);
int midas_gpu_nn_free(midas_gpu_nn *net);
long long midas_gpu_nn_param_count(const midas_gpu_nn *net);
/* set = 0 reads the parameters (grads = 1: the gradients of the last
 * midas_gpu_nn_gradients / train_step) into buf; set = 1 writes them. */
int midas_gpu_nn_params(midas_gpu_ctx *ctx, midas_gpu_nn *net, int set, float *buf, int grads);
int midas_gpu_nn_forward(midas_gpu_ctx *ctx, midas_gpu_nn *net, int batch, const float *inputs, const float *mask,
                         float *E);
/* Loss L = mean over the batch of sum(mask |E_pred - target|^2) / sum(mask |target|^2)
 * and the gradient of every parameter (read them with midas_gpu_nn_params). */
int midas_gpu_nn_gradients(midas_gpu_ctx *ctx, midas_gpu_nn *net, int batch, const float *inputs, const float *mask,
                           const float *target, double *loss);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) at learning rate lr on that loss. */
int midas_gpu_nn_train_step(midas_gpu_ctx *ctx, midas_gpu_nn *net, int batch, const float *inputs, const float *mask,
                            const float *target, float lr, double *loss);

/* The network as a learned right preconditioner (no counterpart in the
 * reference).  The same network, with the 16 input channels holding a cell
 * vector v on the grid: Re, Im of chi in 0-1, s D^-1 v (D = 1 - Znnpp, the
 * Jacobi term) in 2-7, s v in 8-13, the mask in 14 and Re 3 / (eps + 2) in 15,
 * each complex vector as (Re, Im) of x, y, z; the prediction (channels 2-7 plus
 * the network's output, divided by s) approximates Z^-1 v.  The cells must lie
 * on one lattice whose box fits the network's grid; the box is centred in it.
 *
 * midas_gpu_nn_prec_grid writes these inputs and the mask for ncol cell vectors
 * V (3n x ncol column-major complex, host or device) at scales scale[ncol]:
 * the training pairs of the preconditioner (inputs from r = Z e, the target e
 * read from channels 8-13 of the grid of e at r's scale).
 *
 * midas_gpu_fgmres_solve is midas_gpu_gmres_solve with the network as its
 * right preconditioner (flexible GMRES: the preconditioned vectors are kept);
 * convergence is judged on the FP64 true residual as there. */
int midas_gpu_nn_prec_grid(midas_gpu_ctx *ctx, midas_gpu_nn *net, int ncol, const double *V, const double *scale,
                           float *inputs, float *mask);
int midas_gpu_fgmres_solve(midas_gpu_ctx *ctx, midas_gpu_nn *net, int ntr, const double *theta, const double *phi,
                           const double *E0, int restart, int maxit, double tol, double *E, midas_gpu_info *info);

/* Plain MoM: fill, solve, internal field E (3n x 2ntr).  The field part of
 * Compute_EFields_MoM (src/Compute_EFields_MoM.f90:66-229). */
int midas_gpu_mom_solve(midas_gpu_ctx *ctx, int ntr, const double *theta, const double *phi, double *E,
                        midas_gpu_info *info);

/* CBFM-E flags. */
enum midas_cbfm_flags {
    MIDAS_CBFM_SR = 1,      /* threshold the extended-block matrices (SR = 1, the reference default) */
    MIDAS_CBFM_HOMOG = 2,   /* homogeneous scatterer (homogs = 1): PARDISO mtype 6 symmetric storage */
    MIDAS_CBFM_ACA = 4,     /* off-diagonal reduced blocks from ACA factors (Use_ACA = 1) */
    MIDAS_CBFM_FAST_CBF = 8, /* CBF block solves refined with an FP32-grade residual instead of double-float */
    MIDAS_CBFM_SPHERICAL = 16 /* CBF excitations are spherical waves (type_iws = 2/3, Incident_Field_Spherical,
                                 src/Compute_EFields_CBFME.f90:363-368); plane waves (type_iws = 1) otherwise */
};

/* CBFM-E solve: Compute_EFields_CBFME (src/Compute_EFields_CBFME.f90:1-1006) or,
 * with MIDAS_CBFM_ACA, Compute_EFields_CBFME_ACA.
 *   cells are ordered by block: block b owns cells blk_offsets[b]..blk_offsets[b+1]-1;
 *   ext_offsets (nblocks+1) / ext_idx list the extension cells of each block
 *   (CBFM_Blocks_Ext, src/Extend_blocks.f90:134);
 *   ncbf directions (cbf_theta/cbf_phi) are the CBF excitations
 *   (getTransmitters_CBFM, src/getParameters_CBFM.f90:1-110);
 *   thr_cbf is Threshold_CBFM (<= 0: the reference rule of :286-288);
 *   res_sr is res_SR (<= 0: the reference default);
 *   E (3n x 2ntr) receives the internal field, K (nblocks, may be NULL) the CBF counts. */
int midas_gpu_cbfm_solve(midas_gpu_ctx *ctx, int nblocks, const int *blk_offsets, const int *ext_offsets,
                         const int *ext_idx, int ncbf, const double *cbf_theta, const double *cbf_phi,
                         double thr_cbf, double res_sr, int flags, double eps_aca, int aca_itmax, int ntr,
                         const double *theta, const double *phi, double *E, int *K, midas_gpu_info *info);

/* Extinction and absorption cross sections from the internal field
 * (Compute_ExtAbsCsec_fromIntField, src/Compute_ExtAbsCsec_fromIntField.f90:45-64). */
int midas_gpu_cext_cabs(midas_gpu_ctx *ctx, int ntr, const double *theta, const double *phi, const double *E,
                        double *cext, double *cabs);
/* Far-field scattering matrix, nrx x 4ntr (Vv, Vh, Hv, Hh per direction):
 * GetFFieldCoeff + projection (src/Green_functions.f90:1399-1438,
 * src/Compute_EFields_MoM.f90:306-369). */
int midas_gpu_smatrix(midas_gpu_ctx *ctx, int nrx, const double *rx_theta, const double *rx_phi, int ntr,
                      const double *E, double *S);

/* Integration rules of the incident (transmitter) and scattering (receiver)
 * direction sets: NumIntType_t / NumIntType_r (src/InOut_ReadWrite_Functions.f90:319). */
enum midas_quad {
    MIDAS_QUAD_UN = 0,   /* uniform theta x phi grid, adaptive quadrature ('un') */
    MIDAS_QUAD_TR = 1,   /* uniform grid, trapezoid cubature ('tr') */
    MIDAS_QUAD_GL = 2,   /* Gauss-Legendre grid, caller's weights ('gl') */
    MIDAS_QUAD_SD = 3,   /* spherical design list, equal weights ('sd') */
    MIDAS_QUAD_LB = 4,   /* Lebedev list, caller's weights ('lb') */
    MIDAS_QUAD_RF = 5    /* directions read from a file, equal weights ('rf') */
};

/* Efficiencies per incident direction and their orientation averages:
 * Compute_Scattering_Quantities_1 (grid transmitters 'un' / 'tr' / 'gl') and
 * Compute_Scattering_Quantities_2 (transmitter lists 'sd' / 'rf' / 'lb'),
 * src/Compute_Scattering_Quantities.f90:1-1012, with the reference's grid-sampled
 * QUADPACK QAG (src/quadpack.f90, src/Numerical_Integration.f90:213-305).
 *   Transmitters: ntr_theta x ntr_phi directions (degrees, theta fastest; a list
 *   has ntr_phi = 1).  Receivers: nrx_theta x nrx_phi directions (a list: nrx_phi
 *   = 1) followed by extra receivers up to nrx_tot (the forward and backward
 *   directions, get_trans_Receiv, src/get_trans_Receiv.f90:506-600).
 *   S: nrx_tot x 4ntr complex, column-major, Vv, Vh, Hv, Hh per transmitter (the
 *   layout of midas_gpu_smatrix); cext / cabs: per transmitter
 *   (midas_gpu_cext_cabs).  dm: the scatterer's diameter (X = k0 dm / 2).
 *   cext_intfields: CextIntFields (1 = Q_ext from the internal field).
 *   w_tr / w_rx: 'gl' theta weights then phi weights, 'lb' one per direction,
 *   else NULL.
 *   q_dir (5 x ntr): Q_ext, Q_abs, Q_sca, Q_bks, g per transmitter (the Qidtable
 *   columns); q_avg (5): the same averaged over the transmitters (the qtable).
 * Every array may live in host or device memory.  A forward or backward
 * direction missing from the receivers, or an 'un' grid whose samples fall
 * outside it (the reference's index map needs theta and phi ranges that start
 * at 0), returns MIDAS_ERR_ARG. */
int midas_gpu_scattering_quantities(midas_gpu_ctx *ctx, int quad_tr, int quad_rx, int ntr_theta, int ntr_phi,
                                    const double *tr_theta, const double *tr_phi, int nrx_theta, int nrx_phi,
                                    int nrx_tot, const double *rx_theta, const double *rx_phi, const double *S,
                                    const double *cext, const double *cabs, double dm, double k0, int cext_intfields,
                                    const double *w_tr, const double *w_rx, double *q_dir, double *q_avg);

/* Dense complex solve that allocates no device memory (no counterpart in the
 * reference).  For callers that cannot call cudaMalloc: plug-ins whose host
 * application owns and caps all device memory, and latency-critical paths where
 * an allocation could block.  It solves A X = B (A n x n, B n x nrhs,
 * column-major complex, host or device memory; B is overwritten by X) with the
 * same mixed-precision LU + FP64 refinement as midas_gpu_dense_solve, on
 * `stream` (a cudaStream_t; NULL = the legacy default stream) of `device`.
 * No context is needed.  All scratch comes from one static 24 MiB device array
 * inside the library, which every GPU that loads the library holds until exit;
 * a scratch request beyond it returns MIDAS_ERR_ALLOC, never a cudaMalloc.
 * Limits: n <= 512, nrhs <= 32 (larger sizes return MIDAS_ERR_ARG).  All calls
 * share the array: calls that overlap on the GPU race, so serialise them.  The
 * call is synchronous (it waits on `stream` and reads the refinement's
 * convergence on the host); on a stream that is being captured it returns
 * MIDAS_ERR_ARG without issuing work.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress) and caches it.
 * *backward_error (may be NULL) receives the final normwise backward error. */
int midas_gpu_dense_solve_noalloc(int device, void *stream, int n, int nrhs, const double *A, double *B,
                                  double *backward_error);

/* Diagnostics (no counterpart in the reference). */
/* Device self-test of the tensor-core GEMM engine against a CUDA-core GEMM on a
 * ragged problem; returns MIDAS_OK when they agree to TF32 accuracy. */
int midas_gpu_gemm_selftest(midas_gpu_ctx *ctx);
/* Name of the GEMM engine in use ("tcgen05"). */
const char *midas_gpu_gemm_engine(void);
/* Check of the bounded device waits: one kernel waits, with `limit` polls
 * (1..2^20), on an mbarrier that nothing arrives at, through the same wait
 * routine as the tensor-core kernels.  The wait expires, *expired is set to 1 and
 * the call returns MIDAS_ERR_DEVICE_TIMEOUT; the context stays usable. */
int midas_gpu_wait_selftest(midas_gpu_ctx *ctx, int limit, int *expired);
/* Hermitian eigen-decomposition on the device (the CBF singular-value step):
 * A is m x m row-major complex; W receives the eigenvalues in descending order and
 * V (row-major m x m) the eigenvectors as columns. */
int midas_gpu_heev(midas_gpu_ctx *ctx, int m, const double *A, double *W, double *V);
/* FP32-grade complex product D = A B on the tensor cores (the split-TF32 GEMM of
 * the reduced-matrix assembly); A (M x K), B (K x N), D (M x N) row-major complex. */
int midas_gpu_zgemm_x3(midas_gpu_ctx *ctx, int M, int N, int K, const double *A, const double *B, double *D);
/* Average device time (CUDA events on the context stream) of `iters` launches of
 * the tensor-core GEMM D[M x N] -= A[M x K] Bt[N x K]^T on internal buffers (fp32). */
int midas_gpu_bench_gemm(midas_gpu_ctx *ctx, int M, int N, int K, int iters, double *ms);
/* The same with fp16 operands (the kind::f16 path of the LU trailing update) when
 * f16 != 0; D stays fp32. */
int midas_gpu_bench_gemm_ex(midas_gpu_ctx *ctx, int M, int N, int K, int iters, int f16, double *ms);
/* Number of kernels this context has launched so far. */
long long midas_gpu_launch_count(const midas_gpu_ctx *ctx);
/* The context's CUDA stream (a cudaStream_t): every kernel of the context runs on it. */
void *midas_gpu_stream(const midas_gpu_ctx *ctx);
/* Stream ordering without a host wait (the asynchronous form of the boundary; no
 * counterpart in the reference, whose calls are blocking).  midas_gpu_wait_event
 * makes all work the context issues after it -- its own stream, and the CBFM lanes,
 * which start from that stream -- wait for `event` (a cudaEvent_t the caller
 * recorded, e.g. after producing device-resident inputs on its own stream).
 * midas_gpu_record_event records `event` (a cudaEvent_t) on the context stream
 * after the work issued so far, for a caller's stream to wait on.  The solve entry
 * points themselves return when their results are complete: the refinement reads
 * its convergence test on the host. */
int midas_gpu_wait_event(midas_gpu_ctx *ctx, void *event);
int midas_gpu_record_event(midas_gpu_ctx *ctx, void *event);

/* Kernel classes timed by the profiler below. */
#define MIDAS_KC_GEMM_TC   0   /* tcgen05 GEMM: LU trailing-matrix updates (and untagged GEMMs) */
#define MIDAS_KC_GEMM_SIMT 1   /* CUDA-core FP32 GEMM (fallback engine) */
#define MIDAS_KC_FILL      2   /* impedance fills (MoM element, CBFM block, SR threshold) */
#define MIDAS_KC_SR_SCAN   3   /* setfSR ladder scan */
#define MIDAS_KC_DIAG_LU   4   /* diagonal-block LU and inverses */
#define MIDAS_KC_TRSV      5   /* blocked triangular solves */
#define MIDAS_KC_RESID     6   /* refinement residuals (FP64 / double-float) */
#define MIDAS_KC_ZGEMM64   7   /* FP64 complex GEMMs (Gram, CBF projections, Vc, E) */
#define MIDAS_KC_EIG       8   /* Hermitian eigensolver */
#define MIDAS_KC_OTHER     9   /* everything else that is instrumented (ACA) */
#define MIDAS_KC_GEMM_PANEL 10  /* tcgen05 GEMM: LU panel and U-row (forward substitution) steps */
#define MIDAS_KC_GEMM_SOLVE 11  /* tcgen05 GEMM: triangular-solve updates */
#define MIDAS_KC_GEMM_PROD  12  /* tcgen05 GEMM: split-TF32 products (reduced matrix, FP32-grade ZGEMM) */
#define MIDAS_KC_SPLIT      13  /* split-TF32 operand preparation (hi / lo pieces) */
#define MIDAS_KC_LATTICE   14  /* FFT lattice operator (scatter, FFTs, spectral product, gather) */
#define MIDAS_KC_NN        15  /* tcgen05 GEMMs of the learned initial guess's convolutions */
#define MIDAS_KC_RESID32   16  /* FP32 residual updates r -= Z d of the refinements */
#define MIDAS_KC_COUNT     17
/* enable = 1 clears the per-class totals and starts timing every instrumented
 * launch with CUDA events on the context stream; 0 stops.  Timing adds one event
 * record before and after each instrumented launch. */
int midas_gpu_profile(midas_gpu_ctx *ctx, int enable);
/* Totals of one kernel class since profiling was enabled: device milliseconds,
 * algorithmic flops and bytes (the op's own counts, not hardware counters) and
 * launches.  Waits for the recorded events. */
int midas_gpu_profile_query(midas_gpu_ctx *ctx, int kclass, double *ms, double *flops, double *bytes,
                            long long *launches);

#ifdef __cplusplus
}
#endif
#endif /* MIDAS_GPU_H */
