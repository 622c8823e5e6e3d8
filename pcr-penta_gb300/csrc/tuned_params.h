// tuned_params.h -- defaults chosen by the autotuner (pcrp/autotune.py) on NVIDIA GB300.
// Regenerated by `python -m pcrp.autotune --write`; edit there, not here.
#pragma once
#define PCRP_TUNED_SMEM_ROWS 512     // ragged path: shared-memory capacity (rows)
#define PCRP_TUNED_FUSE_STRIDES 2     // ragged path: strides fused per global pass
#define PCRP_TUNED_TILE_ROWS 500      // ragged path: rows written per CTA in a global pass
#define PCRP_TUNED_THREADS 256        // threads per CTA
#define PCRP_TUNED_MP_SMEM_BLOCKS 1024   // mixed: block rows solved whole in shared memory
#define PCRP_TUNED_MP_FUSE 5            // mixed: FP32 block strides fused per global pass
// FP64 path by system size: {n_max, smem_rows, fuse_strides, tile_rows, threads}
#define PCRP_TUNED_F64_TABLE { \
    {512, 512, 3, 484, 256}, \
    {1024, 512, 3, 484, 256}, \
    {8192, 512, 2, 500, 256}, \
    {131072, 512, 1, 508, 256}, \
    {2097152, 512, 2, 500, 256} }
// mixed path by system size: {n_max, block rows in shared memory, fuse_strides}
#define PCRP_TUNED_MP_TABLE { \
    {1024, 2048, 2}, \
    {8192, 1024, 5}, \
    {131072, 1024, 5}, \
    {2097152, 1024, 5} }
