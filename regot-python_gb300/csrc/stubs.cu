// Temporary: solvers not built yet.
#include "solvers.h"
namespace regot {
#define STUB(NAME) void NAME(regot_ctx*, regot_dproblem*, double, double, int, const regot_opts&, regot_result*) { throw Error(REGOT_ERR_INVALID_ARG, #NAME " is not available yet"); }
STUB(sinkhorn_ssns_gpu)
}
