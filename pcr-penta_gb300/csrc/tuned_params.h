// tuned_params.h -- defaults chosen by the autotuner (pcrp/autotune.py).
// Regenerated by `python -m pcrp.autotune --write`; edit there, not here.
#pragma once
#define PCRP_TUNED_SMEM_ROWS 1024     // largest subsystem solved whole in shared memory
#define PCRP_TUNED_FUSE_STRIDES 3     // PCR strides fused per global pass
#define PCRP_TUNED_TILE_ROWS 996      // rows written per CTA in a global pass
#define PCRP_TUNED_THREADS 256        // threads per CTA
