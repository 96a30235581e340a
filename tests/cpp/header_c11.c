/* The C-ABI header compiled as C11: every declaration must be plain C. */
#include "rrea_gpu.h"

#include <stddef.h>

_Static_assert(sizeof(rrea_gpu_config) == 136, "rrea_gpu_config layout");
_Static_assert(sizeof(rrea_gpu_secondary) == 112, "rrea_gpu_secondary layout");
_Static_assert(offsetof(rrea_gpu_secondary, birth_fraction) == 104, "rrea_gpu_secondary tail");
_Static_assert(offsetof(rrea_gpu_seed_event, weight) == 80, "rrea_gpu_seed_event tail");

rrea_gpu_status rrea_c11_probe(rrea_gpu_ctx* ctx)
{
    rrea_gpu_config cfg;
    rrea_gpu_default_config(&cfg);
    (void)cfg;
    return rrea_gpu_reset_sources(ctx);
}
