// cages_harness.cpp -- one-rank restatement of the host side of
// cuda_build_cages (src/cuda_particle.cu:1516-1646) around the reference's
// unmodified cage kernels (src/particle_kernel.cu:79-576: reset_flag_*,
// reset_phases, cage_setup, build_phase, build_phase_shell, cage_flag_*,
// flag_external_*), compiled for the CPU with emu_cuda.h.  Test
// infrastructure: it produces the fixtures the oracle's and the drop-in's cage
// builders are checked against.  It uses the domain, BC and launch shapes
// ref_setup (harness.cpp) prepared.
#include <cstdint>
#include <cstring>
#include <vector>

extern "C" {
#include "bluebottle.h"
#include "bluebottle.cuh"
}
#include "cuda_particle.h"

extern dom_struct DOM;
extern BC bc;

static int threads2(int n) { return n < MAX_THREADS_DIM ? n : MAX_THREADS_DIM; }
static int cdiv(int a, int b) { return (a + b - 1) / b; }

// Particles as (x, y, z, r) rows in domain coordinates; with_parts = NPARTS > 0.
// Outputs are the reference's ghosted arrays: phase and phase_shell (Gcc s3b),
// flag_u, flag_v, flag_w (Gfx, Gfy, Gfz s3b).
extern "C" int ref_build_cages(int with_parts, int np, const double *xyzr, int *phase_out, int *shell_out,
                               int *fu_out, int *fv_out, int *fw_out) {
  dom_struct &d = dom[0];
  const grid_info &G = d.Gcc;
  std::vector<part_struct> parts(np > 0 ? np : 1);
  memset(parts.data(), 0, sizeof(part_struct) * parts.size());
  for (int n = 0; n < np; n++) {
    parts[n].N = n;
    parts[n].x = xyzr[4 * n + 0];
    parts[n].y = xyzr[4 * n + 1];
    parts[n].z = xyzr[4 * n + 2];
    parts[n].r = xyzr[4 * n + 3];
  }
  // launch shapes of cuda_blocks_init for the ghosted extents
  const dim3 fx_dim(threads2(d.Gfx.jnb), threads2(d.Gfx.knb)), fx_num(cdiv(d.Gfx.jnb, threads2(d.Gfx.jnb)),
                                                                       cdiv(d.Gfx.knb, threads2(d.Gfx.knb)));
  const dim3 fy_dim(threads2(d.Gfy.knb), threads2(d.Gfy.inb)), fy_num(cdiv(d.Gfy.knb, threads2(d.Gfy.knb)),
                                                                       cdiv(d.Gfy.inb, threads2(d.Gfy.inb)));
  const dim3 fz_dim(threads2(d.Gfz.inb), threads2(d.Gfz.jnb)), fz_num(cdiv(d.Gfz.inb, threads2(d.Gfz.inb)),
                                                                       cdiv(d.Gfz.jnb, threads2(d.Gfz.jnb)));
  const dim3 cc_dim(threads2(G.inb), threads2(G.jnb)), cc_num(cdiv(G.inb, threads2(G.inb)),
                                                               cdiv(G.jnb, threads2(G.jnb)));
  emu::launch(fx_num, fx_dim, [&] { reset_flag_u(_flag_u); });
  emu::launch(fy_num, fy_dim, [&] { reset_flag_v(_flag_v); });
  emu::launch(fz_num, fz_dim, [&] { reset_flag_w(_flag_w); });
  NPARTS = with_parts;
  nparts = np;
  if (with_parts > 0) {
    emu::launch(cc_num, cc_dim, [&] { reset_phases(_phase, _phase_shell); });
    const int tx = (int)(0.5 * MAX_THREADS_DIM), ty = tx, tz = tx;
    const real itx = 1. / tx, ity = 1. / ty, itz = 1. / tz;
    int cage_dim[3];
    for (int pass = 0; pass < 2; pass++)
      for (int n = 0; n < np; n++) {
        emu::launch(dim3(1), dim3(1), [&] { cage_setup(parts.data(), n, cage_dim); });
        const int bx = (int)ceil((real)cage_dim[0] * itx);
        const int by = (int)ceil((real)cage_dim[1] * ity);
        const int bz = (int)ceil((real)cage_dim[2] * itz);
        if (bx > 0 && by > 0 && bz > 0) {
          if (pass == 0)
            emu::launch(dim3(bx, by, bz), dim3(tx, ty, tz),
                        [&] { build_phase(parts.data(), n, cage_dim, _phase, _phase_shell, &DOM, &bc); });
          else
            emu::launch(dim3(bx, by, bz), dim3(tx, ty, tz),
                        [&] { build_phase_shell(parts.data(), n, cage_dim, _phase, _phase_shell, &DOM, &bc); });
        }
      }
    emu::launch(fx_num, fx_dim, [&] { cage_flag_u(_flag_u, _phase, _phase_shell); });
    emu::launch(fy_num, fy_dim, [&] { cage_flag_v(_flag_v, _phase, _phase_shell); });
    emu::launch(fz_num, fz_dim, [&] { cage_flag_w(_flag_w, _phase, _phase_shell); });
  }
  // one rank: it is the first and the last subdomain in every direction
  if (bc.pW != PERIODIC && bc.pE != PERIODIC) {
    emu::launch(fx_num, fx_dim, [&] { flag_external_u(_flag_u, d.Gfx._is); });
    emu::launch(fx_num, fx_dim, [&] { flag_external_u(_flag_u, d.Gfx._ie); });
  }
  if (bc.pS != PERIODIC && bc.pN != PERIODIC) {
    emu::launch(fy_num, fy_dim, [&] { flag_external_v(_flag_v, d.Gfy._js); });
    emu::launch(fy_num, fy_dim, [&] { flag_external_v(_flag_v, d.Gfy._je); });
  }
  if (bc.pB != PERIODIC && bc.pT != PERIODIC) {
    emu::launch(fz_num, fz_dim, [&] { flag_external_w(_flag_w, d.Gfz._ks); });
    emu::launch(fz_num, fz_dim, [&] { flag_external_w(_flag_w, d.Gfz._ke); });
  }
  memcpy(phase_out, _phase, sizeof(int) * G.s3b);
  memcpy(shell_out, _phase_shell, sizeof(int) * G.s3b);
  memcpy(fu_out, _flag_u, sizeof(int) * d.Gfx.s3b);
  memcpy(fv_out, _flag_v, sizeof(int) * d.Gfy.s3b);
  memcpy(fw_out, _flag_w, sizeof(int) * d.Gfz.s3b);
  return 0;
}

// sizeof(part_struct) of this build (-DDOUBLE): the stride of _parts
extern "C" long long ref_part_struct_bytes(void) { return (long long)sizeof(part_struct); }
