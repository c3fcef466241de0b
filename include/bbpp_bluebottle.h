/*
 * bbpp_bluebottle.h -- drop-in replacement of the Bluebottle pressure solve.
 *
 * libbbpp_bluebottle.so exports the three functions the Bluebottle time loop
 * calls (src/bluebottle.c:139,228-232,393-395) with the reference's
 * signatures.  They read the same globals the reference solver reads
 * (defined by the host program in src/bluebottle.c:438-576 and
 * src/cuda_bluebottle.cu:34-35) and write the same output (_phi), so a
 * Bluebottle build links this library in place of src/cuda_solver.cu and
 * src/solver_kernel.cu.  One rank, one GPU: nprocs must be 1 (the halo
 * exchange is replaced by on-device periodic wrap).
 *
 * The struct layouts below repeat the reference's (src/domain.h:52-94,
 * 168-210; src/bluebottle.h:662) member for member, because the library
 * reads the host program's objects of these types.
 */
#ifndef BBPP_BLUEBOTTLE_H
#define BBPP_BLUEBOTTLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef double bb_real; /* the reference's `real` with -DDOUBLE (src/bluebottle.h:45-51) */

/* grid_info, src/domain.h:52-94 */
typedef struct bb_grid_info {
  int is, ie, in, isb, ieb, inb;
  int js, je, jn, jsb, jeb, jnb;
  int ks, ke, kn, ksb, keb, knb;
  int _is, _ie, _isb, _ieb;
  int _js, _je, _jsb, _jeb;
  int _ks, _ke, _ksb, _keb;
  int s1, s1b, s2, s2b, s3, s3b;
  int s2_i, s2_j, s2_k, s2b_i, s2b_j, s2b_k;
} bb_grid_info;

/* dom_struct, src/domain.h:168-210 */
typedef struct bb_dom_struct {
  bb_grid_info Gcc, Gfx, Gfy, Gfz;
  bb_real xs, xe, xl;
  int xn;
  bb_real dx;
  bb_real ys, ye, yl;
  int yn;
  bb_real dy;
  bb_real zs, ze, zl;
  int zn;
  bb_real dz;
  int rank;
  int e, w, n, s, t, b;
  int I, Is, Ie, In;
  int J, Js, Je, Jn;
  int K, Ks, Ke, Kn;
  int S1, S2, S3;
} bb_dom_struct;

/* The leading members of BC (src/bluebottle.h:662-668); the solver reads
 * only the pressure boundary types. */
typedef struct bb_bc_pressure {
  int pW, pE, pS, pN, pB, pT;
} bb_bc_pressure;

/* The leading members of part_struct (src/particle.h:343-348) and its size
 * with -DDOUBLE and the reference's NNODES 26, MAX_COEFFS 15, S_MAX_COEFFS 25
 * and MAX_NEIGHBORS 12 (src/particle.h:42-83): the cage builder reads each
 * particle's radius and centre from the host program's device array _parts,
 * whose stride is that size. */
#define BB_PART_STRUCT_BYTES 3128
typedef struct bb_part_head {
  int N;
  bb_real r, x, y, z;
} bb_part_head;

/* ---- entry points (src/bluebottle.h:3073,3085,3112; defined in the
 * reference at src/cuda_solver.cu:31,38,573) ---- */

/* Re-derive the solver's view of the particles after the cages were rebuilt:
 * the one-byte phase mask (solid = _phase > -1) and _invM
 * (PP_jacobi_init, src/solver_kernel.cu:26-87). */
void cuda_PP_init_jacobi_preconditioner(void);
/* Pressure solve with particles (src/cuda_solver.cu:38-300): rhs from
 * u*,v*,w* (PP_rhs), cuda_part_BC_p(), coeffs_refine, Jacobi PCG from phi = 0
 * until (r,z) <= pp_residual^2 (rhs,rhs), phi written to _phi's interior,
 * one row appended through recorder_PP.  NaN residual or more than
 * pp_max_iter iterations print the reference's messages and exit(EXIT_FAILURE). */
void cuda_PP_cg(void);
/* The same without particles (src/cuda_solver.cu:573-761). */
void cuda_PP_cg_noparts(void);
/* Per-phase timed variant (src/cuda_solver.cu:302-571): the same solve with
 * kernel timing on; writes recorder_PP_timed rows to solver_expd_timed.rec.
 * The search-direction update and both dot products are fused into the two
 * solver kernels, so spmv holds the fused SpMV kernel, up1 the fused update
 * kernel (plus residual replacements), and ip1/ar1/ip2/ar2/up2/mpi are 0. */
void cuda_PP_cg_timed(void);

/* The time loop's steps after the solve (src/bluebottle.c:233-252), same names and
 * signatures as src/cuda_bluebottle.cu:2495-2589, one rank:
 *  cuda_dom_BC_p(array): Neumann ghost planes of a cell array = the adjacent interior
 *    cells (periodic ghosts are the host's mpi_cuda_exchange_Gcc);
 *  cuda_project(): u, v, w = u*, v*, w* - dt/rho_f |flag| grad(_phi) on every face;
 *  cuda_update_p(): _p = (fluid) (_p0 + _phi) on the interior, minus its mean over all cells.
 * All launch on the default stream, as the reference's. */
void cuda_dom_BC_p(bb_real *array);
void cuda_project(void);
void cuda_update_p(void);

/* The phase field and face flags of the particles' cages, same name and
 * signature as src/cuda_particle.cu:1516 (declared src/cuda_particle.h), one
 * rank: flags reset to 1; with particles (NPARTS > 0) _phase = the index of the
 * last particle whose sphere contains the cell centre (else -1), _phase_shell
 * = 0 on solid cells with a face neighbour outside their particle (else 1), and
 * the face flags -1 across a phase change or between two shell cells; 0 on
 * both wall faces of a non-periodic direction.  Reads _parts[0 .. nparts-1]
 * (the host program's particles, periodic copies included, as the reference's
 * kernels do).  Six launches on the default stream, whatever nparts. */
void cuda_build_cages(void);

/* Free the library's private device workspace (no counterpart in the
 * reference, whose solver uses the host program's buffers). */
void bbpp_bluebottle_release(void);

/* ---- globals read from the host program ----
 * Declared for the library's own translation unit only: a Bluebottle source
 * file includes src/bluebottle.h, which declares the same objects with the
 * reference's type names and already declares the entry points above. */
#ifdef BBPP_BLUEBOTTLE_IMPL
extern bb_dom_struct *dom;
extern int rank, nprocs;
extern int NPARTS, nparts;
extern bb_real rho_f, dt;
extern bb_real pp_residual;
extern int pp_max_iter;
extern int stepnum;
extern bb_real *_phi, *_rhs_p, *_invM;
extern bb_real *_u_star, *_v_star, *_w_star;
extern int *_phase;
extern bb_real *_u, *_v, *_w, *_p, *_p0;  /* the epilogue's fields */
extern int *_flag_u, *_flag_v, *_flag_w;
extern int *_phase_shell;
extern unsigned char *_parts; /* part_struct *, read at stride BB_PART_STRUCT_BYTES */
/* ---- functions of the host program the solver calls ---- */
void cuda_part_BC_p(void);                                              /* src/cuda_particle.cu:1679 */
void recorder_PP(char *name, int niter, bb_real resid, bb_real etime);  /* src/recorder.c:190 */
void recorder_PP_init_timed(char *name);                                /* src/recorder.c:223 */
void recorder_PP_timed(char *name, int niter, bb_real resid, bb_real etime, bb_real etime_spmv,
                       bb_real etime_ip1, bb_real etime_AR1, bb_real etime_up1, bb_real etime_ip2,
                       bb_real etime_AR2, bb_real etime_up2, bb_real etime_mpi); /* src/recorder.c:263 */
#endif /* BBPP_BLUEBOTTLE_IMPL */

#ifdef __cplusplus
}
#endif
#endif
