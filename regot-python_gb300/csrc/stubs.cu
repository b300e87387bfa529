// Temporary: solvers not built yet.
#include "solvers.h"
namespace regot {
#define STUB(NAME) void NAME(regot_ctx*, regot_dproblem*, double, double, int, const regot_opts&, regot_result*) { throw Error(REGOT_ERR_INVALID_ARG, #NAME " is not available yet"); }
STUB(sinkhorn_newton_gpu)
STUB(sinkhorn_ssns_gpu)
STUB(qrot_lbfgs_dual_gpu)
STUB(qrot_assn_gpu)
}
extern "C" {
int regot_qrot_dual_obj_grad(regot_ctx*, regot_dproblem*, double, const double*, double*, double*) { return REGOT_ERR_INVALID_ARG; }
int regot_qrot_optimal_beta(regot_ctx*, regot_dproblem*, double, const double*, double*) { return REGOT_ERR_INVALID_ARG; }
int regot_qrot_primal_val(regot_ctx*, regot_dproblem*, double, const double*, double*) { return REGOT_ERR_INVALID_ARG; }
int regot_qrot_plan(regot_ctx*, regot_dproblem*, double, const double*, double*, int) { return REGOT_ERR_INVALID_ARG; }
}
