// bbpp_net.cu -- learned initial guess (placeholder until the network
// kernels land): returns BBPP_BAD_ARG.
#include "bbpp_internal.h"

int bbpp_net_guess(bbpp_ctx *ctx, void *net, const uint8_t *mask, const double *rhs, const double *prev, double *x,
                   double *ms) {
  (void)ctx;
  (void)net;
  (void)mask;
  (void)rhs;
  (void)prev;
  (void)x;
  if (ms) *ms = 0;
  return BBPP_BAD_ARG;
}

void bbpp_net_ctx_free(bbpp_ctx *ctx) { (void)ctx; }
