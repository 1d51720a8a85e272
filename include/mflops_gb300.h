/*
 * mflops_gb300.h -- C ABI of the GB300 (sm_103a) implementation of the
 * MFLOPS3D-MD hot path: compact finite-difference derivatives, the
 * matrix-diagonalisation Poisson/Helmholtz solver, the spline filter and
 * the influence-matrix multidomain coupling.
 *
 * Conventions
 *  - Every function returns an int status (MF_OK = 0); mf_last_error()
 *    returns a thread-local description of the last failure.  No function
 *    calls exit() and no device code traps.
 *  - 3D arrays are FP64, Fortran (column-major) order: f(i,j,k) lives at
 *    f[i + nx*(j + ny*k)], x fastest, exactly the memory of the reference's
 *    real(rk) :: f(nx,ny,nz).  Coefficient tables exported by the set-up
 *    functions are Fortran-ordered too (dl(n,5) -> dl[i + n*m]).
 *  - Field pointers may be HOST or DEVICE memory; the library inspects each
 *    pointer.  Host pointers are staged through device buffers owned by the
 *    handle and the call returns after the result is back in host memory.
 *    Of a host solution array (solve_3d's solf) only the 12 edge lines go
 *    to the device: the solve writes its interior and faces, and the edges
 *    come back unchanged, as in the reference.
 *    Device-pointer calls are asynchronous on `stream` (a cudaStream_t, NULL
 *    for the legacy default stream).
 *  - A handle may be used by one host thread at a time; distinct handles
 *    are independent.
 */
#ifndef MFLOPS_GB300_H
#define MFLOPS_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define MF_OK 0
#define MF_ERR_ARG 1           /* bad argument, shape or size              */
#define MF_ERR_COMPLEX_EIG 2   /* 1D operator has complex eigenvalues       */
#define MF_ERR_SINGULAR 3      /* singular small/dense system in set-up     */
#define MF_ERR_CUDA 4          /* CUDA runtime error                        */
#define MF_ERR_TIMEOUT 5       /* a bounded device wait expired             */
#define MF_ERR_NOT_CONVERGED 6 /* iteration limit reached                   */
#define MF_ERR_ALLOC 7         /* device allocation failed                  */
#define MF_ERR_UNSUPPORTED 8   /* size/mode outside what the kernels support */

/* Precision modes of the solver transforms. */
#define MF_PREC_FP64 0        /* plain FP64 (drop-in, matches the reference)       */
#define MF_PREC_SPLIT_BF16 1  /* split-BF16 three-product on tcgen05, FP32 accum.  */
#define MF_PREC_3XTF32 2      /* 3xTF32 on tcgen05, FP32 accumulation              */

/* Arithmetic of the FP64-accurate refinement residual of the mixed path
 * (tridiagonal second-derivative operators): FP64 sweeps (default) or
 * double-FP32 throughout (error-free products and sums on the FP32 pipe).
 * Both evaluate the cancelling stencil sums in moment form. */
#define MF_RESID_FF 0
#define MF_RESID_FP64 1       /* FP64 sweeps; two lanes per line (twisted factorisation) on the y, z passes */
#define MF_RESID_FP64_LINE 2  /* FP64 sweeps, one thread per line */

const char* mf_last_error(void);

/* Launch-shape autotuner (no reference counterpart).  mode 0 (default):
 * built-in heuristics; mode 1: the first call for a problem shape times the
 * candidate launch shapes (FP64 transform tiles 32 or 64; staged or strided
 * x-line derivative sweeps) with CUDA events on the caller's stream, keeps
 * the fastest and reuses it (no timing while a stream is being captured, and
 * none for in-place derivative calls).  The candidates give identical
 * results.  Decisions can be saved to and loaded from a text file. */
int mf_tune_set(int mode);
int mf_tune_get(void);
int mf_tune_entries(void);
int mf_tune_clear(void);
int mf_tune_save(const char* path);
int mf_tune_load(const char* path);
/* Slice width of the 3xTF32 tensor-core transform (no reference
 * counterpart): 0 the default (128-column slices with the matrix streamed
 * through the TMA ring wherever the padded axis is a multiple of 128, or,
 * with mf_tune_set(1), the faster plan measured per shape), 1 64-column
 * slices with the matrix resident in shared memory, 2 128-column slices
 * where possible.  Both plans give identical results.  Process-wide. */
int mf_tc_tf32_plan_set(int plan);
int mf_tc_tf32_plan_get(void);
int mf_version(void);
/* 1 when a CUDA device is usable from this process, else 0. */
int mf_device_available(void);

/* ------------------------------------------------------------------------
 * Host-only set-up routines (no GPU needed).
 * ---------------------------------------------------------------------- */

/* 1D grids of src/class_mesh/class_mesh.f90 (type mesh_grid, grid1d):
 * n nodes on [xa, xb].  kind MF_GRID_UNIFORM: xa + i*pas.  MF_GRID_ARCSIN:
 * the grid mesh_grid_init builds (:181-200), x = xa + (xb-xa)*
 * (asin(-alpha*cos(pi*(xi-xa)/(xb-xa)))/asin(alpha) + 1)/2 with
 * alpha = 1 - param/n^2 (the reference's param is beta = 33.3).
 * MF_GRID_TANH: the tanh stretching of :203, x = xa + (xb-xa)*
 * (1 + tanh(param*(2*(xi-xa)/(xb-xa) - 1))/tanh(param))/2 (param 0 gives
 * the uniform grid).  xi = xa + i*(xb-xa)/(n-1). */
#define MF_GRID_UNIFORM 0
#define MF_GRID_ARCSIN 1
#define MF_GRID_TANH 2
int mf_grid1d(int kind, int n, double xa, double xb, double param, double* grid);

/* dgrid1d of mesh_grid_init (class_mesh.f90:268-276): one-sided spacing at
 * the two ends, centred half-differences inside. */
int mf_grid_spacing(int n, const double* grid, double* dgrid);

/* mesh_grid_init(grid, choice, nx, ny, nz, mpid), class_mesh.f90:113-339:
 * the interval of direction choice ('x', 'y': [-0.5, 0.5]; 'z':
 * [-0.25, 0.25]), cut into ndomains equal slabs of which slab dom_coord is
 * taken (the md_mpi_getcoord / md_mpi_getnumberdomains part, :157-170),
 * then grid1d(n) of the given kind and, if dgrid1d is not NULL, its
 * spacing.  The reference always builds MF_GRID_ARCSIN with param 33.3.
 * The 3-D copies grid3d/dgrid3d are broadcasts of grid1d; callers that
 * need them broadcast the 1D arrays.  derivatives_coefficients_init and
 * solver_init_3d (:316-386) pass grid1d on to mf_der_coeffs_init and
 * mf_solver_coeffs_init_3d. */
int mf_mesh_grid_init(char choice, int n, int dom_coord, int ndomains, int kind, double param,
                      double* grid1d, double* dgrid1d);

/* One row of the compact scheme; replaces der_coeffs_generic of
 * src/class_derivatives/class_derivatives_coefficient.f90:31-191. */
int mf_der_coeffs_generic(const double h0[7], int cl, int der, int so,
                          double coef_imp[5], double coef_exp[7]);

/* dl(n,5) and dr(n,7) of a whole line, NOT factored; replaces
 * der_coeffs_generic_gobal, src/class_derivatives/class_derivatives.f90:330-377. */
int mf_der_line_coeffs(const double* grid, int n, int der, int so, double* dl, double* dr);

/* In-place quasi-pentadiagonal LU of dl(n,5); replaces pentalu,
 * src/class_derivatives/class_derivatives.f90:379-423. */
int mf_pentalu(int n, double* dl);

/* One axis of the solver set-up; replaces solver_coeffs_init,
 * src/class_solver/class_solver_3d.f90:413-466.  grid has nall nodes,
 * n = nall-2.  Outputs (any may be NULL): ddl(n,5), ddr(n,8),
 * inv_lhs(n,n), eigen(n), vect(n,n), inv_vect(n,n), neum(2,7); all
 * Fortran-ordered, vect untransposed (eigenvectors in columns). */
int mf_solver_axis_setup(const double* grid, int nall, const int bct[2], int so,
                         double* ddl, double* ddr, double* inv_lhs, double* eigen,
                         double* vect, double* inv_vect, double* neum);

/* ------------------------------------------------------------------------
 * Compact derivatives: type(derivatives_coefficients)
 * ---------------------------------------------------------------------- */
typedef struct mf_der mf_der_t;

/* der_coeffs_init(grid,dc,n,solve,so), src/class_derivatives/class_derivatives.f90:111-184.
 * solver_type != 0 also builds the n-2 "solver type" coefficient set. */
int mf_der_coeffs_init(const double* grid, int n, int solver_type, int so, mf_der_t** dc);
int mf_der_destroy(mf_der_t* dc);
/* dertype(dc), class_derivatives.f90:96-109 */
int mf_dertype(const mf_der_t* dc, int* solver_type);

/* Field-level pencil drivers derx, dery, derz, dderx, ddery, dderz of
 * src/class_field/class_field.f90:629-978: df = d/dx_axis^order of f along
 * `axis` (0=x,1=y,2=z), order 1 or 2.  f, df are (nx,ny,nz).  With a
 * solver-type dc, the pencils on the two boundary faces normal to the other
 * axes use der_s/dder_s (interior n-2 points, end values 0) and the four
 * edge lines are 0. */
int mf_der_apply(const mf_der_t* dc, int axis, int order, const double* f, double* df,
                 int nx, int ny, int nz, void* stream);
int mf_derx(const mf_der_t* dc, const double* f, double* df, int nx, int ny, int nz, void* stream);
int mf_dery(const mf_der_t* dc, const double* f, double* df, int nx, int ny, int nz, void* stream);
int mf_derz(const mf_der_t* dc, const double* f, double* df, int nx, int ny, int nz, void* stream);
int mf_dderx(const mf_der_t* dc, const double* f, double* df, int nx, int ny, int nz, void* stream);
int mf_ddery(const mf_der_t* dc, const double* f, double* df, int nx, int ny, int nz, void* stream);
int mf_dderz(const mf_der_t* dc, const double* f, double* df, int nx, int ny, int nz, void* stream);

/* `count` (1..9) sweeps of mf_der_apply in one launch: job q differentiates
 * f[q] along axis[q] (order[q] 1 or 2) with dc[q] into df[q]; all fields are
 * (nx,ny,nz) device arrays and df[q] must not alias any f.  The results equal
 * those of separate mf_der_apply calls.  No reference counterpart: it puts
 * the lines of independent sweeps of a small field into one grid. */
int mf_der_apply_many(int count, const mf_der_t* const* dc, const int* axis, const int* order,
                      const double* const* f, double* const* df, int nx, int ny, int nz, void* stream);

/* Single-pencil forms der/dder/der_s/dder_s (class_derivatives.f90:186-260)
 * on `count` contiguous pencils of length n (x[p*n + i]). */
int mf_der_lines(const mf_der_t* dc, int order, int solver_variant, const double* x, double* dx,
                 int count, void* stream);

/* ------------------------------------------------------------------------
 * Matrix-diagonalisation solver: type(solver_coeffs_3d)
 * ---------------------------------------------------------------------- */
typedef struct mf_solver3d mf_solver3d_t;

/* solver_coeffs_init_3d(grid1,grid2,grid3,sc,n1,n2,n3,bct,so),
 * src/class_solver/class_solver_3d.f90:380-411.  n1,n2,n3 are the node
 * counts INCLUDING the two boundary nodes (grid1(n1) ...).
 * bct = (x1,x2,y1,y2,z1,z2), 1 Dirichlet / 2 Neumann / 3 second derivative. */
int mf_solver_coeffs_init_3d(const double* grid1, const double* grid2, const double* grid3,
                             int n1, int n2, int n3, const int bct[6], int so,
                             mf_solver3d_t** sc);
int mf_solver3d_destroy(mf_solver3d_t* sc);

/* solve_3d(sc,rhs,sigma,solf,bcx,bcy,bcz,n1,n2,n3),
 * src/class_solver/class_solver_3d.f90:83-299, plain FP64.
 * Here n1,n2,n3 are INTERIOR counts: rhs(n1,n2,n3), solf(0:n1+1,0:n2+1,0:n3+1),
 * bcx(n2,n3,2), bcy(n1,n3,2), bcz(n1,n2,2).  Solves
 * (Lx+Ly+Lz+sigma) u = rhs; writes the interior and the six faces of solf
 * (edges/corners untouched).  Unlike the reference, rhs is not modified. */
int mf_solve_3d(mf_solver3d_t* sc, const double* rhs, double sigma, double* solf,
                const double* bcx, const double* bcy, const double* bcz,
                int n1, int n2, int n3, void* stream);

/* Allocation-free variant of mf_solve_3d (plain FP64), with no counterpart
 * in the reference.  It is for callers that cannot let a library call
 * cudaMalloc: applications whose device memory belongs to their own pool
 * allocator, which budgets every byte and forbids other allocations, and
 * latency-bound host loops that cannot afford cudaMalloc's implicit
 * device-wide synchronisation.  Its two work arrays live in a fixed 4 MiB
 * file-scope device array, so the interior n1*n2*n3 is limited to 262144
 * points (64^3); larger sizes return MF_ERR_UNSUPPORTED.  All pointers must
 * be device memory (MF_ERR_ARG otherwise).  The first call on each device
 * looks up that array's address with cudaGetSymbolAddress (no allocation).
 * Every call shares the array, so calls that overlap on the GPU (different
 * streams or handles) race; each call overwrites the work arrays before
 * reading them.  It calls no cudaMalloc, cudaFree or allocating library
 * routine. */
int mf_solve_3d_noalloc(mf_solver3d_t* sc, const double* rhs, double sigma, double* solf,
                        const double* bcx, const double* bcy, const double* bcz,
                        int n1, int n2, int n3, void* stream);

/* `count` problems of this operator and sigma (plain FP64) in one pass of
 * launches: problem b reads rhs + b*rhs_stride and the boundary arrays at
 * b times their strides, and writes solf + b*solf_stride (element strides;
 * a stride of 0 shares one input array between all problems).  Each
 * problem's result equals that of mf_solve_3d.  Device pointers only,
 * 1 <= count <= 65535.  No reference counterpart (the reference solves one
 * right-hand side per solve_3d call); used for the influence-matrix columns
 * and for several right-hand sides of one operator. */
int mf_solve_3d_batch(mf_solver3d_t* sc, int count, const double* rhs, long long rhs_stride,
                      double sigma, double* solf, long long solf_stride, const double* bcx,
                      long long bcx_stride, const double* bcy, long long bcy_stride,
                      const double* bcz, long long bcz_stride, int n1, int n2, int n3,
                      void* stream);

/* Same problem with the eigenvector transforms on the tensor cores
 * (precision = MF_PREC_SPLIT_BF16 or MF_PREC_3XTF32) and `refine`
 * iterative-refinement steps whose residual is computed in FP64 with the
 * solver's own compact operator.  refine < 0 selects the default count. */
int mf_solve_3d_mixed(mf_solver3d_t* sc, const double* rhs, double sigma, double* solf,
                      const double* bcx, const double* bcy, const double* bcz,
                      int n1, int n2, int n3, int precision, int refine, void* stream);

/* `count` problems through mf_solve_3d_mixed (precision MF_PREC_FP64: the
 * plain solve) in one call, with host (pinned for overlap) or device arrays
 * given per problem: the upload of problem b+1 and the download of problem
 * b-1 run on copy streams while problem b is solved (three device staging
 * slots).  In the mixed modes every problem after the first of a call is
 * one replay of its slot's CUDA graph, captured on first use and again
 * when sigma, the precision, the refinement count, the transform plan, the
 * tuner mode or the residual form change, or after mf_solver3d_set_eigen
 * (not while the per-kernel timers of mf_solver3d_profile are on).  Each problem's result equals that of a
 * single call; the call returns when every result is in place.  No
 * reference counterpart (the reference solves one right-hand side per
 * call). */
int mf_solve_3d_mixed_many(mf_solver3d_t* sc, int count, const double* const* rhs, double sigma,
                           double* const* solf, const double* const* bcx, const double* const* bcy,
                           const double* const* bcz, int n1, int n2, int n3, int precision,
                           int refine, void* stream);

/* class_field::solver_3d(sc,g,u,bc,sigma), src/class_field/class_field.f90:1072-1109:
 * g,u are (nx,ny,nz) fields (nx = n1+2 ...); the interior of g is the
 * right-hand side and the result is written into u. */
int mf_solver_3d(mf_solver3d_t* sc, const double* g, double* u,
                 const double* bcx, const double* bcy, const double* bcz,
                 int nx, int ny, int nz, double sigma, int precision, void* stream);

/* Replaces the eigen-decomposition of one axis (0=x,1=y,2=z) with
 * caller-supplied tables: eigen(n), vect(n,n) (eigenvectors in columns) and
 * inv_vect(n,n), Fortran-ordered and untransposed -- e.g. the LAPACK dgeev
 * output that solver_matrix_init computes (class_solver_3d.f90:535-564).
 * The solve is invariant to the choice of eigenvector basis, but operators
 * with a null eigenvalue (bct = 3 next to Dirichlet, all-Neumann) amplify the
 * basis' rounding; loading the caller's tables makes the results follow the
 * caller's decomposition.  Synchronous; device or host pointers. */
int mf_solver3d_set_eigen(mf_solver3d_t* sc, int axis, const double* eigen, const double* vect,
                          const double* inv_vect);

/* Selects the residual arithmetic (MF_RESID_FP64, default; MF_RESID_FP64_LINE;
 * MF_RESID_FF) used by the mixed solves of this handle; no counterpart in
 * the reference. */
int mf_solver3d_set_residual(mf_solver3d_t* sc, int mode);
/* Reads and clears the device-side error flag of the tensor-core pipeline
 * (MF_ERR_TIMEOUT if a bounded wait expired since the last call). Syncs. */
int mf_solver3d_device_status(mf_solver3d_t* sc);

/* Per-kernel CUDA-event timers of a solver handle (stage timers in the
 * spirit of the reference's cpu_time/MPI_WTIME stage prints,
 * class_solver_3d.f90:106-259, class_field.f90:1317-1386).  profile(sc,1)
 * resets and enables, profile(sc,0) disables.  profile_read syncs and
 * returns the accumulated time and kernel launch count of one stage:
 * 0 tensor-core transform (split store), 1 residual x pass, 2 residual y/z passes,
 * 3 FP64 residual narrowed to the operand (with the null-mode projection
 * of closed operators), 4 boundary fold (with its face products), 5 boundary faces,
 * 6 FP64 transform, 7 interior copy, 8 tensor-core transform with the
 * eigenvalue divide, 9 tensor-core transform updating the FP64 solution,
 * 10 FP32 correction residual. */
int mf_solver3d_profile(mf_solver3d_t* sc, int enable);
int mf_solver3d_profile_read(mf_solver3d_t* sc, int kind, double* total_ms, long long* launches);

/* FP64 residual r = g - (Lx+Ly+Lz+sigma) u on the interior (u with its
 * boundary data bcx/bcy/bcz), all interior-sized (n1,n2,n3).  Device memory. */
int mf_solver_residual(mf_solver3d_t* sc, const double* g, const double* u, double sigma,
                       const double* bcx, const double* bcy, const double* bcz,
                       double* r, int n1, int n2, int n3, void* stream);

/* ------------------------------------------------------------------------
 * Influence-matrix multidomain coupling (class_md + class_field MD driver),
 * every subdomain resident on one GPU.
 * Subdomain (i,j,k) of an nd = (nd1,nd2,nd3) decomposition has index
 * s = i + nd1*(j + nd2*k) and owns the x-grid of slab i, the y-grid of slab j
 * and the z-grid of slab k (conforming faces; neighbours share their
 * interface nodes).  Interface faces are Dirichlet; physical faces use bct.
 * ---------------------------------------------------------------------- */
typedef struct mf_md mf_md_t;

/* Interface numbering of md_influence_matrix_param,
 * src/class_md/class_md.f90:1450-1680 (host only).  nint_x[i] = interior
 * points of x-slab i, etc.  Outputs (any may be NULL): dm_int(nd1,nd2,nd3,3,2)
 * Fortran-ordered (1-based ids, -1 none; side 1 left, 2 right), and per
 * interface its axis (0..2), size (points) and offset (first row); it =
 * number of interfaces, ninf = number of interface unknowns. */
int mf_md_topology(const int nd[3], const int periods[3], const int* nint_x, const int* nint_y,
                   const int* nint_z, int* dm_int, int* kind, int* size, int* offset, int* it,
                   long long* ninf);

/* Creates the subdomain solvers (solver_coeffs_init_3d) and solver-type
 * derivative coefficients (der_coeffs_init) of every subdomain:
 * gridx[i] has nx[i] nodes (i < nd1), gridy[j] ny[j], gridz[k] nz[k];
 * md_bc_init (class_md.f90:275-293) turns interface faces into Dirichlet. */
int mf_md_create(const int nd[3], const int periods[3], const double* const* gridx, const int* nx,
                 const double* const* gridy, const int* ny, const double* const* gridz, const int* nz,
                 const int bct[6], int so, mf_md_t** md);
int mf_md_destroy(mf_md_t* md);
int mf_md_ninf(const mf_md_t* md, long long* ninf, int* it);

/* Builds and factorises the influence matrix for one sigma
 * (influence_matrix_init_end + md_influence_matrix_set,
 * class_field.f90:1216-1287,1396-1510): one Dirac column per interface point,
 * FP64, then an FP64 LU.  null_mode: 0 none, 1 constant null space (rhs and
 * solution made mean-free, as a KSP with a null space), 2 row 0 pinned
 * (md_add_pert / md_vector_zero_lastpoint, class_md.f90:223-268). */
int mf_md_influence_matrix_set(mf_md_t* md, double sigma, int null_mode, void* stream);

/* multidomain_solve(mpid,inf,sc,bc,u,g,du,sigma,dcx,dcy,dcz,null),
 * class_field.f90:1295-1388: per subdomain s, g[s] and u[s] are (nx,ny,nz)
 * fields and bcx[s](ny-2,nz-2,2), bcy[s], bcz[s] the physical boundary data
 * (interface faces ignored).  Device pointers. */
int mf_md_solve(mf_md_t* md, const double* const* g, double* const* u, const double* const* bcx,
                const double* const* bcy, const double* const* bcz, void* stream);
/* multidomain_solve for nrhs (1..4) right-hand sides of the same operator
 * (the reference calls it once per velocity component,
 * class_navier_3D.f90:1643-1648,1699-1704,1753-1758): g, u, bcx, bcy, bcz
 * hold nrhs x (subdomain count) pointers, right-hand side major.  Results
 * equal nrhs calls of mf_md_solve; the interface systems are solved together,
 * one pass over the explicit inverse for all of them. */
int mf_md_solve_many(mf_md_t* md, int nrhs, const double* const* g, double* const* u,
                     const double* const* bcx, const double* const* bcy, const double* const* bcz,
                     void* stream);

/* md_solve (class_md.f90:379-438): the interface system alone for nrhs
 * (1..4) right-hand sides stored one after the other at rhs (ninf each,
 * device), solutions to sol, in the form mf_md_interface_form reports, with
 * the operator's null-space handling (md_rhs_nullspace,
 * md_vector_zero_lastpoint).  mf_md_solve calls the same step between its two
 * rounds of subdomain solves. */
int mf_md_interface_solve(mf_md_t* md, int nrhs, const double* rhs, double* sol, void* stream);

/* Interface-system solve form (no reference counterpart: the reference solves
 * it with a PETSc KSP, class_md.f90:379-438).  MF_MD_IFACE_AUTO (default):
 * when ninf <= 12,000 one FP64 matrix-vector product with the inverse formed
 * at set-up; above, two row-parallel triangular products with the inverted LU
 * factors (MF_MD_IFACE_TRIANGULAR_INVERSE); the triangular solves on the LU
 * factors when neither fits in device memory.  MF_MD_IFACE_LU: always the two
 * triangular solves on the getrf factors.  Takes effect at the next
 * mf_md_solve; the inverse forms are built by mf_md_influence_matrix_set (and
 * mf_md_load_factor), so select the mode before it. */
#define MF_MD_IFACE_AUTO 0
#define MF_MD_IFACE_LU 1
/* MF_MD_IFACE_INVERSE: the inverse at any size when it fits in device memory
 * (2 n^3 FP64 flops at set-up, then one n^2 read per solve; for long runs). */
#define MF_MD_IFACE_INVERSE 2
/* MF_MD_IFACE_TRIANGULAR_INVERSE: the inverted LU factors at any size when
 * they fit (2 n^3 / 3 FP64 flops at set-up, as the getrf; then the same n^2
 * read per solve as MF_MD_IFACE_INVERSE, in two launches).  The factors are
 * stored as double-float pairs (FP32 hi + lo, 8 bytes an entry, scaled by a
 * power of two) and the products run on the FP32 pipe, about 2^-48 relative
 * per term; MF_MD_IFACE_TRIANGULAR_INVERSE_FP64 keeps FP64 entries and FP64
 * FMAs (bound by GB300's FP64 rate, one FMA per 8 bytes read).  A factor with
 * a non-finite entry stays FP64. */
#define MF_MD_IFACE_TRIANGULAR_INVERSE 3
#define MF_MD_IFACE_TRIANGULAR_INVERSE_FP64 4
int mf_md_set_interface_solve(mf_md_t* md, int mode);
/* The form the next solve takes (MF_MD_IFACE_INVERSE, _TRIANGULAR_INVERSE,
 * _TRIANGULAR_INVERSE_FP64 or _LU), after mf_md_influence_matrix_set or
 * mf_md_load_factor. */
int mf_md_interface_form(const mf_md_t* md, int* form);
/* Form of the triangular solves on the LU factors (no reference
 * counterpart): MF_MD_TRI_PERSISTENT (default) one cooperative launch per
 * triangle, CTAs advancing through 64-row blocks behind release/acquire
 * flags (every wait bounded; mf_md_device_status reports an expired one);
 * MF_MD_TRI_STEPS one launch per 128-row block step.  Used also when the
 * persistent form cannot be launched. */
#define MF_MD_TRI_PERSISTENT 0
#define MF_MD_TRI_STEPS 1
int mf_md_set_triangular_form(mf_md_t* md, int form);
/* Synchronises and returns MF_ERR_TIMEOUT if a persistent triangular solve
 * gave up waiting (the results of that solve are then not valid). */
int mf_md_device_status(const mf_md_t* md);
/* Precision of the subdomain solves inside mf_md_solve (MF_PREC_FP64, the
 * default, or a mixed mode with `refine` steps); the influence matrix is
 * FP64 either way. */
int mf_md_set_precision(mf_md_t* md, int precision, int refine);

/* On-disk factor cache (the role of md_influence_matrix_filename / _write /
 * _read, class_md.f90:918-956, which name the cached matrix after the grid
 * sizes only).  The key is a 64-bit FNV-1a hash of everything the matrix
 * depends on -- decomposition, periods, every slab's grid, boundary types,
 * scheme order, sigma and the null mode -- as 16 hex digits.  save writes the
 * LU factor and pivots of the last mf_md_influence_matrix_set; load reads
 * them (MF_ERR_ARG for a file of another key, a truncated or a damaged file)
 * and rebuilds the solve tables; cached loads dir/<key>.mffac when it exists
 * and builds and writes it otherwise. */
int mf_md_factor_key(const mf_md_t* md, double sigma, int null_mode, char key[17]);
int mf_md_save_factor(const mf_md_t* md, const char* path);
int mf_md_load_factor(mf_md_t* md, double sigma, int null_mode, const char* path, void* stream);
int mf_md_influence_matrix_cached(mf_md_t* md, double sigma, int null_mode, const char* dir, void* stream);

/* How mf_md_influence_matrix_set forms the influence columns (no reference
 * counterpart: the reference solves one subdomain problem per Dirac column,
 * class_field.f90:1396-1510).  MF_MD_ASSEMBLY_EIGEN (default): in each
 * subdomain solver's eigenbasis, where a Dirac datum is separable, one
 * face-to-face block of n^5 FP64 work per pair of interface faces.
 * MF_MD_ASSEMBLY_SOLVES: batched subdomain solves of all Dirac columns and
 * derivative sweeps, n^4 work per column.  The two agree to rounding. */
#define MF_MD_ASSEMBLY_EIGEN 0
#define MF_MD_ASSEMBLY_SOLVES 1
int mf_md_set_assembly(mf_md_t* md, int mode);

/* Copies the last interface solution (ninf values) to host memory. */
int mf_md_interface(const mf_md_t* md, double* lambda);

/* ------------------------------------------------------------------------
 * Least-squares B-spline filter (class_filter).  For fixed data sites,
 * weights and knots the fit is a linear operator P (no x ni) shared by every
 * pencil of an axis; P' gives the first derivative.
 * ---------------------------------------------------------------------- */
typedef struct mf_filter mf_filter_t;

/* Operators of LSQUnivariateSpline(ni,xi,yi,wi,nn,xn,no,xo,yo,ypo,k),
 * src/class_filter/class_filter.f90:104-174 (fixed-knot weighted least
 * squares of degree k, knots (k+1)*xi(1), xn(2:nn-1), (k+1)*xi(ni); values
 * and first derivatives at xo).  Host only; P, Pd are (no,ni) Fortran-ordered,
 * either may be NULL; wi may be NULL (unit weights). */
int mf_filter_lsq_matrix(const double* xi, int ni, const double* wi, const double* xn, int nn,
                         const double* xo, int no, int k, double* P, double* Pd);
/* Operators of interp_period(ni,xi,yi,nos,xos,yos), class_filter.f90:267-347
 * (periodic quintic least squares on nn = ni-6 equispaced nodes, evaluated at
 * xos; the last data point only fixes the period).  Host only. */
int mf_filter_period_matrix(const double* xi, int ni, const double* xos, int nos, double* P,
                            double* Pd);
/* Handles holding the operators on the device (filter type + flt_init,
 * class_filter.f90:9-73). */
int mf_filter_lsq_init(const double* xi, int ni, const double* wi, const double* xn, int nn,
                       const double* xo, int no, int k, mf_filter_t** f);
int mf_filter_period_init(const double* xi, int ni, const double* xos, int nos, mf_filter_t** f);
int mf_filter_destroy(mf_filter_t* f);
int mf_filter_matrix(const mf_filter_t* f, int deriv, double* P);
/* Applies the filter (deriv = 0) or its derivative (deriv = 1) along `axis`
 * of an (nx,ny,nz) field whose length along that axis is ni; out has no
 * points along it.  Host or device pointers. */
int mf_filter_apply(const mf_filter_t* f, int axis, int deriv, const double* in, int nx, int ny,
                    int nz, double* out, void* stream);
/* Pencil forms with the reference's signatures (one pencil; GPU apply). */
int mf_lsq_univariate_spline(int ni, const double* xi, const double* yi, const double* wi, int nn,
                             const double* xn, int no, const double* xo, double* yo, double* ypo,
                             int k);
int mf_interp_period(int ni, const double* xi, const double* yi, int nos, const double* xos,
                     double* yos);

/* ------------------------------------------------------------------------
 * LES eddy viscosity: navier_LES, src/class_navier/class_navier_3D.f90:1225-1455
 * (with les_sigma, :1458-1502).  les_type 0 none, 1 Smagorinsky, 2 WALE,
 * 3 sigma model; nu is multiplied by (dx^2+dy^2+dz^2)/3 (one-sided spacing
 * at the ends) and is zero on the twelve edge lines.
 * ---------------------------------------------------------------------- */
typedef struct mf_les mf_les_t;

/* Grids of the three axes (host), as in navier%gridx/gridy/gridz. */
int mf_les_create(const double* gx, int nx, const double* gy, int ny, const double* gz, int nz,
                  mf_les_t** les);
int mf_les_destroy(mf_les_t* les);
/* nu from the nine gradient fields du[3*i+j] = d u_i / d x_j (device, (nx,ny,nz)). */
int mf_les_nu(const mf_les_t* les, int les_type, double c, const double* const* du, double* nu,
              void* stream);
/* Whole navier_LES step from the velocity: the nine first derivatives of
 * u, v, w with the derivative handles of x, y and z (derx/dery/derz), then
 * nu.  Device pointers; the gradients live in scratch owned by `les`. */
int mf_les_nu_velocity(mf_les_t* les, const mf_der_t* dcx, const mf_der_t* dcy,
                       const mf_der_t* dcz, int les_type, double c, const double* u,
                       const double* v, const double* w, double* nu, void* stream);

/* ------------------------------------------------------------------------
 * Channel-flow statistics: src/main/post_prod.f90:40-238 (mean, rms and
 * cross-correlation profiles along y, friction velocity) on nt snapshots of
 * u, v, w, p already in device memory ((nx,ny,nz) each; host grids).
 * Outputs (host): moy[4*ny] = mean u, v, w, p normalised by u_tau (p by
 * u_tau^2); rms[7*ny] = rms u, v, w, p and the uv, uw, vw correlations;
 * *utau.  so: order of the compact derivative used for du/dy at the walls.
 * ---------------------------------------------------------------------- */
int mf_channel_stats(int nt, const double* const* u, const double* const* v, const double* const* w,
                     const double* const* p, int nx, int ny, int nz, const double* gx, const double* gy,
                     const double* gz, double re, int so, double* moy, double* rms, double* utau,
                     void* stream);

/* ------------------------------------------------------------------------
 * Learned LES coefficient.  No reference counterpart: the reference has only
 * the plain models above.  A 6-64-64-1 ReLU network (4,673 FP32 parameters)
 * maps six invariants of the resolved velocity gradient,
 *   S:S/G2, tr(S^3)/G2^1.5, tr(W^2 S)/G2^1.5, tr(W^2 S^2)/G2^2,
 *   det(g)/G2^1.5, tr(g)/G2^0.5            (G2 = g:g),
 * to C(x) in nu_t = C(x) Delta^2 sqrt(2 S:S).  Features and network are FP32.
 * Outside the training range of the features (or where g:g leaves
 * (1e-30, 1e30)) the plain Smagorinsky model is used per point.
 * ---------------------------------------------------------------------- */
typedef struct mf_mlp mf_mlp_t;

/* New network: He-uniform weights from `seed`, zero biases, output bias 1. */
int mf_mlp_create(unsigned long long seed, mf_mlp_t** mlp);
int mf_mlp_destroy(mf_mlp_t* mlp);
/* 4,673: W1[64][6], b1[64], W2[64][64], b2[64], w3[64], b3 (FP32). */
int mf_mlp_num_params(void);
int mf_mlp_get_params(const mf_mlp_t* mlp, float* host_params);
/* Replaces the parameters and resets the Adam moments. */
int mf_mlp_set_params(mf_mlp_t* mlp, const float* host_params);
/* Input standardisation x = (f - mean) * istd, training range [lo, hi] per
 * feature, output scale (C = cscale * network output) and loss scale. */
int mf_mlp_set_scaling(mf_mlp_t* mlp, const float* mean, const float* istd, const float* lo,
                       const float* hi, float cscale, float loss_scale);
/* One training step on n points (device arrays: X (n_all, 6) raw features,
 * base (n_all) = Delta^2 sqrt(2 S:S), target (n_all) eddy viscosity; idx
 * (n, int32, each < n_all) selects the points, or NULL for the first n).
 * Loss L = loss_scale / n * sum (C b - target)^2.  lr > 0 applies one Adam
 * step (beta 0.9/0.999, eps 1e-8); lr = 0 only evaluates.  grad_host (4,673
 * floats) and loss_host receive the gradient and loss before the update when
 * not NULL (the call then synchronises the stream). */
int mf_mlp_train_step(mf_mlp_t* mlp, const float* X, const float* base, const float* target,
                      const int* idx, long long n, float lr, float* grad_host, float* loss_host,
                      void* stream);
/* C for n points of raw features X (device). */
int mf_mlp_predict(const mf_mlp_t* mlp, const float* X, long long n, float* C, void* stream);

/* Features and b for every point of the LES grid from the nine gradient
 * fields (device; zero on the edge lines and where g = 0). */
int mf_les_features(const mf_les_t* les, const double* const* du, float* X, float* base,
                    void* stream);
/* A-priori target from filtered fields: ubar[3] = F(u_i), uu[6] = F(u_i u_j)
 * (00, 01, 02, 11, 12, 22), du = grad(ubar); nu = -tau^d:S / (2 S:S). */
int mf_les_sgs_target(const mf_les_t* les, const double* const* ubar, const double* const* uu,
                      const double* const* du, float* nu_true, void* stream);
/* nu from the network where the features are inside its training range,
 * else Smagorinsky with c_fallback (the value mf_les_nu type 1 gives).
 * n_fallback (host, optional) receives the number of fallback points. */
int mf_les_nu_mlp(mf_les_t* les, const mf_mlp_t* mlp, double c_fallback, const double* const* du,
                  double* nu, long long* n_fallback, void* stream);

/* ------------------------------------------------------------------------
 * Fine-grid box flow that generates the training data (no reference
 * counterpart): pointwise parts of an explicit Runge-Kutta + projection step of a
 * decaying flow in a no-slip box; derivatives and the Neumann Poisson solve
 * come from the entry points above.  Device fields (nx,ny,nz), FP64.
 * ---------------------------------------------------------------------- */
/* out_i = a w_i + b (u_i + dt (nu sum_j ddu[3i+j] - sum_j u_j du[3i+j])),
 * zero on the walls; w may be NULL when a == 0. */
int mf_flow_stage(int nx, int ny, int nz, double nu, double dt, double a, double b,
                  const double* const* u, const double* const* w, const double* const* du,
                  const double* const* ddu, double* const* out, void* stream);
/* rhs (nx-2, ny-2, nz-2) = scale (dudx + dvdy + dwdz) at the interior points. */
int mf_flow_divergence(int nx, int ny, int nz, double scale, const double* dudx, const double* dvdy,
                       const double* dwdz, double* rhs, void* stream);
/* u_i -= dt dphi_i in the interior, 0 on the walls. */
int mf_flow_correct(int nx, int ny, int nz, double dt, double* const* u, const double* const* dphi,
                    void* stream);
/* uu = u_i u_j: 00, 01, 02, 11, 12, 22. */
int mf_flow_products(int nx, int ny, int nz, const double* const* u, double* const* uu, void* stream);
/* u = curl(psi) from dpsi[3i+j] = d psi_i / d x_j, 0 on the walls. */
int mf_flow_curl(int nx, int ny, int nz, const double* const* dpsi, double* const* u, void* stream);

/* ------------------------------------------------------------------------
 * Navier-Stokes time step on one domain (the caller of the derivative and
 * solver entry points): src/main/navier3d.f90:48-274 with
 * src/class_navier/class_navier_3D.f90 -- presolve with the nonlinear terms
 * and the forcing (:1528-1595, 1169-1222, 1043-1167), boundary gradient
 * (:695-791), velocity Helmholtz solves (:1597-1761), pressure-increment
 * Poisson solve (:1764-1845, 342-393), projection (:1847-1959),
 * extrapolation (:2010-2050), slot rotation and the driver's diagnostics
 * (navier3d.f90:120-261) and the LES term (navier_LES :1225-1455, f :1083-1099).
 * Covered: one domain and the multidomain branch (mf_navier_create_md), mapt = 0, pressure types 1 to 4,
 * les_type 0..4, nsubite sub-iterations with the driver's convergence test
 * (testconv, navier3d.f90:366-412).  Velocity Dirichlet and
 * pressure Neumann on all faces; boundary values and sources from the
 * reference's exact solution `sol` (:927-1041, steady: wt = 0).  Fields are
 * (nx,ny,nz) FP64 device arrays, x fastest.
 * ---------------------------------------------------------------------- */
typedef struct mf_navier mf_navier_t;
typedef struct {
  double ts;          /* time step (cmd%ts) */
  double reynolds;    /* cmd%reynolds */
  int nlt;            /* nonlinear form: 0 none, 1 advective, 2 skew-symmetric (reference default 2) */
  int pt;             /* pressure type 1..4 (default 1) */
  int tou;            /* BDF order 1, 2, 3 of the velocity (default 2) */
  int top;            /* pressure extrapolation order + 1 (default 2) */
  int so_solver;      /* so(1), default 6 */
  int so_der;         /* so(2), default 6 */
  int flow_rate;      /* 1: the flow-rate term of f for u (always on in the reference) */
  int nmodes;         /* modes of the exact solution (5 in the reference) */
  int precision;      /* solves: MF_PREC_FP64 (the reference's arithmetic) or a mixed mode */
  int refine;         /* refinement steps of the mixed solves, < 0: default */
  int les_type;       /* 0 none, 1 Smagorinsky, 2 WALE, 3 sigma (default 0), 4 learned (MF_LES_LEARNED) */
  double les_c;       /* cmd%les_c; the model coefficient is its square (default 0) */
  int nsubite;        /* sub-iterations per time step (default 1) */
  const char* md_cache_dir;  /* several subdomains: directory of the influence-matrix factor cache, or NULL */
  int md_interface;   /* several subdomains: MF_MD_IFACE_* of the interface solves (default AUTO) */
} mf_navier_params_t;
/* Fills the reference's defaults (command_line.f90:14-35). */
int mf_navier_defaults(mf_navier_params_t* p);
/* navier_initialization (class_navier_3D.f90:2084-2345), one domain: host
 * grids, all fields zero, time 0. */
int mf_navier_create(const double* gx, int nx, const double* gy, int ny, const double* gz, int nz,
                     const mf_navier_params_t* p, mf_navier_t** out);
/* The multidomain branch (mpid%dims /= 0: several subdomains and/or periodic
 * directions, navier_initialization :2100-2272): nd subdomains per axis
 * with gridx[i] (nx[i] nodes) ..., as mf_md_create; the velocity and phi
 * solves go through multidomain_solve (mf_md_solve, FP64; the velocity
 * influence matrix at sigmau, the pressure one at sigma 0 with the constant
 * null space), built at creation (or read from p->md_cache_dir).  Sums of
 * the flow-rate term, diagnostics and testconv run over all subdomains;
 * subdomain s = i + nd1 (j + nd2 k). */
int mf_navier_create_md(const int nd[3], const int periods[3], const double* const* gridx, const int* nx,
                        const double* const* gridy, const int* ny, const double* const* gridz, const int* nz,
                        const mf_navier_params_t* p, mf_navier_t** out);
int mf_navier_subdomains(const mf_navier_t* nav, int* count);
/* Per-subdomain field access (the functions without _sub use subdomain 0). */
int mf_navier_sub_field(mf_navier_t* nav, int sub, int var, int level, double** ptr);
int mf_navier_sub_set_field(mf_navier_t* nav, int sub, int var, int level, const double* f, void* stream);
int mf_navier_sub_get_field(mf_navier_t* nav, int sub, int var, int level, double* f, void* stream);
int mf_navier_destroy(mf_navier_t* nav);
/* Field var (0..4 = u, v, w, p, phi) of time level `level` (0 = it(1), the
 * slot the next step writes, ..., 3 = it(nt), the newest): device pointer,
 * or a copy from / to host or device memory. */
int mf_navier_field(mf_navier_t* nav, int var, int level, double** ptr);
int mf_navier_set_field(mf_navier_t* nav, int var, int level, const double* f, void* stream);
int mf_navier_get_field(mf_navier_t* nav, int var, int level, double* f, void* stream);
/* One time step: navier_time, then per sub-iteration the step and (diag !=
 * NULL) the driver's diagnostics of level it(nt), which remove the weighted
 * mean of that level's pressure (diag holds the last sub-iteration's), then
 * the slot rotation.  diag[12] = div V; V error,
 * relative, time-accumulated; P error, relative, time-accumulated; kinetic
 * energy; P and V stationarity (value, relative).  Without diag the step
 * makes no host synchronisation (capturable in a CUDA graph once the
 * nonlinear-term cache is warm, e.g. after nt steps; a capture of nt steps
 * returns the slots to the same order). */
int mf_navier_step(mf_navier_t* nav, double* diag, void* stream);
/* Simulated time and the flow-rate state (debit, g; 0 before the first step). */
int mf_navier_state(mf_navier_t* nav, double* time, double* debit, double* g);
/* les_type 4 (MF_LES_LEARNED, no reference counterpart): the eddy viscosity
 * of navier_LES comes from the learned coefficient, nu = C(x) Delta^2
 * sqrt(2 S:S) with C from the network (mf_les_nu_mlp, on the same nine
 * gradients the LES stage computes), and from Smagorinsky with les_c^2
 * wherever the features leave the network's training range.  The network
 * stays owned by the caller and must outlive the steps that use it. */
#define MF_LES_LEARNED 4
int mf_navier_set_les_network(mf_navier_t* nav, const mf_mlp_t* mlp);
/* Sub-iterations made by the last step (1 when nsubite = 1; with nsubite > 1
 * the step stops when testconv passes, which synchronises the host once per
 * sub-iteration). */
int mf_navier_subiterations(const mf_navier_t* nav, int* n);
/* Checkpoint of the whole state (restart_write / restart_read,
 * class_navier_3D.f90:186-340, as one raw binary file instead of a NetCDF
 * directory): time, slot order, every level's fields, the right-hand-side
 * history and the flow-rate state, so that a run resumed from it continues
 * bit-identically.  load needs a handle of the same grids; it returns
 * MF_ERR_ARG for another grid or a damaged file. */
int mf_navier_save(mf_navier_t* nav, const char* path, void* stream);
int mf_navier_load(mf_navier_t* nav, const char* path, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MFLOPS_GB300_H */
