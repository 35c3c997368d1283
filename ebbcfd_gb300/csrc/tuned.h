// Generated by ebbcfd_gb300/autotune.py: per-kernel device time on the 1000000-cell seeded
// wedge, both precision forms, for each minimum number of resident blocks per SM
// requested through __launch_bounds__ (1 = the compiler's register choice).
// split k_cell: 6 blocks 38.1 us, 8 blocks 30.5 us, 10 blocks 35.8 us, 12 blocks 38.9 us
// split k_flux: 10 blocks 21.9 us, 12 blocks 19.8 us, 16 blocks 20.2 us, 20 blocks 21.9 us
// split k_update: 4 blocks 30.2 us, 6 blocks 24.8 us, 8 blocks 22.6 us
// fp64 k_cell: 1 blocks 709.1 us, 5 blocks 701.1 us, 6 blocks 704.7 us, 8 blocks 750.8 us
// fp64 k_flux: 1 blocks 710.3 us, 5 blocks 713.0 us, 6 blocks 714.6 us, 8 blocks 722.2 us
// fp64 k_update: 1 blocks 143.5 us, 2 blocks 143.4 us, 3 blocks 143.0 us, 4 blocks 143.1 us
#pragma once
#ifndef EBB_CELL_TB_F
#define EBB_CELL_TB_F 128
#endif
#ifndef EBB_FLUX_TB_F
#define EBB_FLUX_TB_F 128
#endif
#ifndef EBB_CELL_TB_D
#define EBB_CELL_TB_D 128
#endif
#ifndef EBB_FLUX_TB_D
#define EBB_FLUX_TB_D 128
#endif
#ifndef EBB_UPD_TB
#define EBB_UPD_TB 256
#endif
#ifndef EBB_CELL_MINB_F
#define EBB_CELL_MINB_F 8
#endif
#ifndef EBB_FLUX_MINB_F
#define EBB_FLUX_MINB_F 12
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
#define EBB_UPD_MINB_D 3
#endif
