// Adjoint Westervelt: gradients of a focal loss with respect to phased-array
// element phases and amplitudes.
#include "bd_internal.h"

using namespace bd;

extern "C" {

bd_status bd_westervelt_adjoint(bd_context* ctx, const bd_grid* grid, const bd_medium* medium, const bd_source* source,
                                const bd_westervelt_params* params, const bd_focal_loss* loss, double* loss_out,
                                double* grad_phase, double* grad_amp, double* timings_ms) {
    return guard([&] {
        (void)ctx; (void)grid; (void)medium; (void)source; (void)params; (void)loss; (void)loss_out;
        (void)grad_phase; (void)grad_amp; (void)timings_ms;
        fail(BD_ERR_UNSUPPORTED, "bd_westervelt_adjoint is not implemented in this build");
    });
}

}  // extern "C"
