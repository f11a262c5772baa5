// Multigrid preconditioner (placeholder until the hierarchy is built).
#include "model.h"

namespace eqc {
struct MGHier {};
void mg_build(Handle& h) { (void)h; }
void mg_destroy(Handle& h) { delete h.mg; h.mg = nullptr; }
void mg_apply64(Handle&, const double*, double*) { throw Error(EQC_E_STATE, "multigrid not built"); }
void mg_apply32(Handle&, const float*, float*) { throw Error(EQC_E_STATE, "multigrid not built"); }
}  // namespace eqc
