// Generated by ebbcfd_gb300/autotune.py: per-kernel device time on the 1000000-cell seeded
// wedge, both precision forms, for each minimum number of resident blocks per SM
// requested through __launch_bounds__ (1 = the compiler's register choice).
// split k_cell: 8 blocks 40.4 us, 10 blocks 39.0 us, 12 blocks 49.5 us, 14 blocks 57.7 us
// split k_flux: 10 blocks 26.7 us, 12 blocks 24.1 us, 16 blocks 22.6 us, 20 blocks 26.7 us
// split k_update: 4 blocks 43.8 us, 6 blocks 34.5 us, 8 blocks 30.1 us
// fp64 k_cell: 1 blocks 871.1 us, 5 blocks 866.7 us, 6 blocks 868.4 us, 8 blocks 920.8 us
// fp64 k_flux: 1 blocks 706.9 us, 5 blocks 709.5 us, 6 blocks 711.4 us, 8 blocks 716.2 us
// fp64 k_update: 1 blocks 181.7 us, 2 blocks 182.2 us, 3 blocks 153.9 us, 4 blocks 145.7 us
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
