// Generated by ebbcfd_gb300/autotune.py: per-kernel device time of the FP32
// kernels on the 1000000-cell seeded wedge (split precision) for each minimum number
// of resident blocks per SM requested through __launch_bounds__.
// k_cell: 8 blocks 39.7 us, 10 blocks 39.5 us, 12 blocks 50.6 us, 14 blocks 58.3 us
// k_flux: 10 blocks 27.7 us, 12 blocks 24.7 us, 16 blocks 23.4 us, 20 blocks 27.7 us
// k_update: 4 blocks 44.9 us, 6 blocks 35.0 us, 8 blocks 30.8 us
#pragma once
#ifndef EBB_CELL_MINB_F
#define EBB_CELL_MINB_F 10
#endif
#ifndef EBB_FLUX_MINB_F
#define EBB_FLUX_MINB_F 16
#endif
#ifndef EBB_UPD_MINB_F
#define EBB_UPD_MINB_F 8
#endif
