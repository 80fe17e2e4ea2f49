// Entry points whose device implementations are still being written report
// TTG_ERR_UNSUPPORTED instead of computing anything.
#include "ttg_common.cuh"

extern "C" int ttg_dmaxvol(ttg_ctx* c, ttg_int, ttg_int, const double*, ttg_int*, double*, double,
                           ttg_int) {
  if (!c) return TTG_ERR_ARG;
  c->last_error = "maxvol: not built yet";
  return TTG_ERR_UNSUPPORTED;
}

