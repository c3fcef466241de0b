/*
 * host_stub.c -- a minimal stand-in for the Bluebottle host program, for the
 * drop-in tests: it defines the globals the pressure solve reads
 * (src/bluebottle.c:438-576, src/cuda_bluebottle.cu:34-35 for the solver's
 * subset), the part_BC_p effect on the rhs (solid rhs = 0,
 * src/particle_kernel.cu:1753) and recorders that keep the last row.
 * Device arrays are set by the test through these globals.
 */
#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>

#include "bbpp_bluebottle.h"

bb_dom_struct *dom = 0;
bb_bc_pressure bc; /* the solver reads only the leading pressure types of BC */
int rank = 0, nprocs = 1, NPARTS = 0, nparts = 0, stepnum = 1, pp_max_iter = 20000;
bb_real rho_f = 1.0, dt = 1.0, pp_residual = 1e-8;
bb_real *_phi = 0, *_rhs_p = 0, *_invM = 0, *_u_star = 0, *_v_star = 0, *_w_star = 0;
int *_phase = 0;
bb_real *_u = 0, *_v = 0, *_w = 0, *_p = 0, *_p0 = 0; /* the epilogue's fields */
int *_flag_u = 0, *_flag_v = 0, *_flag_w = 0;
int *_phase_shell = 0;         /* the cage builder's outputs */
unsigned char *_parts = 0;     /* device part_struct array, BB_PART_STRUCT_BYTES per particle */

int stub_niter = -1, stub_calls = 0, stub_timed_calls = 0, stub_init_timed = 0;
bb_real stub_resid = -1, stub_etime = -1, stub_spmv = -1, stub_up1 = -1;
char stub_name[256];

void recorder_PP(char *name, int niter, bb_real resid, bb_real etime) {
  strncpy(stub_name, name, sizeof(stub_name) - 1);
  stub_niter = niter;
  stub_resid = resid;
  stub_etime = etime;
  stub_calls++;
}

void recorder_PP_init_timed(char *name) { (void)name; stub_init_timed++; }

void recorder_PP_timed(char *name, int niter, bb_real resid, bb_real etime, bb_real etime_spmv, bb_real etime_ip1,
                       bb_real etime_AR1, bb_real etime_up1, bb_real etime_ip2, bb_real etime_AR2,
                       bb_real etime_up2, bb_real etime_mpi) {
  (void)etime_ip1; (void)etime_AR1; (void)etime_ip2; (void)etime_AR2; (void)etime_up2; (void)etime_mpi;
  strncpy(stub_name, name, sizeof(stub_name) - 1);
  stub_niter = niter;
  stub_resid = resid;
  stub_etime = etime;
  stub_spmv = etime_spmv;
  stub_up1 = etime_up1;
  stub_timed_calls++;
}

/* host-side copy of the phase field, used to zero the solid rhs */
static int *h_phase = 0;
static long long h_n = 0;
void stub_set_phase_host(int *p, long long n) { h_phase = p; h_n = n; }

void cuda_part_BC_p(void) {
  /* solid cells (phase > -1) get a zero rhs; done on the host for simplicity */
  if (!h_phase || !_rhs_p) return;
  static double *buf = 0;
  static long long cap = 0;
  if (cap < h_n) { buf = (double *)realloc(buf, sizeof(double) * h_n); cap = h_n; }
  cudaMemcpy(buf, _rhs_p, sizeof(double) * h_n, cudaMemcpyDeviceToHost);
  for (long long c = 0; c < h_n; c++)
    if (h_phase[c] > -1) buf[c] = 0.;
  cudaMemcpy(_rhs_p, buf, sizeof(double) * h_n, cudaMemcpyHostToDevice);
}
