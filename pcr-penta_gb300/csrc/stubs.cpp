// stubs.cpp -- entry points whose implementation is not built yet.
#include "pcrp_internal.h"
using namespace pcrp;
extern "C" {
pcrp_status pcrp_solve_mixed(const double*, const double*, const double*, const double*, const double*, double*,
                             int64_t, int64_t, int32_t, double, int32_t, const pcrp_opts*, pcrp_stream,
                             pcrp_mixed_info*)
{ return set_error(PCRP_ENOTSUP, "pcrp_solve_mixed: not built"); }
pcrp_status pcrp_residual_f64(const double*, const double*, const double*, const double*, const double*,
                              const double*, const double*, double*, int64_t, int64_t, int32_t, pcrp_stream)
{ return set_error(PCRP_ENOTSUP, "pcrp_residual_f64: not built"); }
pcrp_status pcrp_solve_ragged(const double*, const double*, const double*, const double*, const double*, double*,
                              const int64_t*, int64_t, int64_t, int32_t, double, int32_t, const pcrp_opts*, pcrp_stream)
{ return set_error(PCRP_ENOTSUP, "pcrp_solve_ragged: not built"); }
}
