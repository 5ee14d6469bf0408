// Box-constrained QP solvers (placeholder factories until the kernels land).
#include "abi_util.cuh"
#include "solver.cuh"

namespace ugpu {
std::unique_ptr<Solver> make_mprgp(Context *) { throw Error(UGPU_ERR_UNSUPPORTED, "MPRGP not built yet"); }
std::unique_ptr<Solver> make_pgs(Context *) { throw Error(UGPU_ERR_UNSUPPORTED, "PGS not built yet"); }
}  // namespace ugpu
