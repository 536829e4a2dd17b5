/*
 * wfe_internal.h -- entry points shared between the library's translation
 * units, not exported through the C ABI.
 */
#ifndef WFE_INTERNAL_H
#define WFE_INTERNAL_H

#include <stdint.h>

#include "wfe.h"

namespace wfe {

/* wfe_create with the slab budgets (bytes) of the two CTA-per-pair tiers;
 * 0 keeps the defaults (2 GiB for the shared-memory wavefront tier, 8 GiB
 * for the global-wavefront tier). */
int create_context(const wfe_config* cfg, uint64_t budget5, uint64_t budget6, wfe_ctx** out);

/* WFE_ERR_CUDA once if a tier launch made on the device failed since the
 * last call (its pairs were left unaligned), else WFE_OK.  Call after the
 * work in question has completed. */
int take_launch_error(wfe_ctx* ctx);

}  // namespace wfe

#endif
