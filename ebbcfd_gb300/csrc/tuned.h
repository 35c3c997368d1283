// Generated by ebbcfd_gb300/autotune.py: per-kernel device time on the 1000000-cell seeded
// wedge, both precision forms, for each minimum number of resident blocks per SM
// requested through __launch_bounds__ (1 = the compiler's register choice).
// split k_cell: 8 blocks 41.0 us, 10 blocks 39.3 us, 12 blocks 49.7 us, 14 blocks 57.8 us
// split k_flux: 10 blocks 26.7 us, 12 blocks 24.7 us, 16 blocks 22.6 us, 20 blocks 26.7 us
// split k_update: 4 blocks 44.9 us, 6 blocks 34.9 us, 8 blocks 30.7 us
// fp64 k_cell: 1 blocks 710.1 us, 5 blocks 702.5 us, 6 blocks 706.2 us, 8 blocks 755.6 us
// fp64 k_flux: 1 blocks 712.1 us, 5 blocks 715.2 us, 6 blocks 716.0 us, 8 blocks 722.3 us
// fp64 k_update: 1 blocks 182.6 us, 2 blocks 182.6 us, 3 blocks 155.6 us, 4 blocks 145.5 us
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
#ifndef EBB_CELL_MINB_D
#define EBB_CELL_MINB_D 5
#endif
#ifndef EBB_FLUX_MINB_D
#define EBB_FLUX_MINB_D 1
#endif
#ifndef EBB_UPD_MINB_D
#define EBB_UPD_MINB_D 4
#endif
