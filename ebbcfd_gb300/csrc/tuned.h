// Generated by ebbcfd_gb300/autotune.py on the default-size plate workload: device time per
// launch of each kernel of the three precision forms for each (threads per block) x (minimum
// resident blocks per SM requested through __launch_bounds__; 1 = the compiler's
// register choice), best of three rounds of CUDA-event timing; fastest kept.
// split k_cell: 64x12 136.8 us, 64x16 146.4 us, 128x6 137.6 us, 128x8 146.6 us, 128x10 167.6 us, 256x3 138.0 us, 256x4 149.1 us
// split k_flux: 64x16 133.5 us, 64x20 123.8 us, 128x8 134.8 us, 128x10 124.9 us, 128x12 115.7 us, 256x4 149.1 us, 256x6 119.7 us
// split k_update: 256x4 135.4 us, 256x6 137.6 us, 256x8 149.9 us, 512x2 140.3 us, 512x3 143.8 us, 512x4 156.5 us
// fp64 k_cell: 64x8 2823.6 us, 64x10 2807.1 us, 128x1 2822.2 us, 128x5 2806.9 us, 128x6 2803.7 us, 256x2 2838.4 us, 256x3 2816.8 us
// fp64 k_flux: 64x6 5267.0 us, 64x8 5267.6 us, 128x1 5268.1 us, 128x4 5268.3 us, 128x5 5340.1 us, 256x1 5286.7 us, 256x2 5285.4 us
// fp64 k_update: 256x1 662.5 us, 256x2 662.3 us, 256x3 566.2 us, 256x4 566.1 us, 512x1 761.0 us, 512x2 604.2 us
// df k_cell: 64x4 1098.1 us, 64x6 1095.0 us, 128x1 1080.5 us, 128x2 1080.5 us, 128x3 1079.8 us, 256x1 1041.0 us, 256x2 1039.7 us
// df k_flux: 64x4 1162.8 us, 64x6 1162.0 us, 128x1 1150.5 us, 128x2 1150.9 us, 128x3 1152.3 us, 256x1 1447.1 us, 256x2 1048.4 us
// df k_update: 256x1 361.8 us, 256x2 361.9 us, 256x3 360.4 us, 256x4 317.4 us, 512x1 553.8 us, 512x2 350.9 us
// update block size 256 (summed best update times: 256: 1018.9 us, 512: 1095.5 us)
#pragma once
#ifndef EBB_CELL_TB_F
#define EBB_CELL_TB_F 64
#endif
#ifndef EBB_CELL_MINB_F
#define EBB_CELL_MINB_F 12
#endif
#ifndef EBB_FLUX_TB_F
#define EBB_FLUX_TB_F 128
#endif
#ifndef EBB_FLUX_MINB_F
#define EBB_FLUX_MINB_F 12
#endif
#ifndef EBB_CELL_TB_D
#define EBB_CELL_TB_D 128
#endif
#ifndef EBB_CELL_MINB_D
#define EBB_CELL_MINB_D 6
#endif
#ifndef EBB_FLUX_TB_D
#define EBB_FLUX_TB_D 64
#endif
#ifndef EBB_FLUX_MINB_D
#define EBB_FLUX_MINB_D 6
#endif
#ifndef EBB_CELL_TB_W
#define EBB_CELL_TB_W 256
#endif
#ifndef EBB_CELL_MINB_W
#define EBB_CELL_MINB_W 2
#endif
#ifndef EBB_FLUX_TB_W
#define EBB_FLUX_TB_W 256
#endif
#ifndef EBB_FLUX_MINB_W
#define EBB_FLUX_MINB_W 2
#endif
#ifndef EBB_UPD_TB
#define EBB_UPD_TB 256
#endif
#ifndef EBB_UPD_MINB_F
#define EBB_UPD_MINB_F 4
#endif
#ifndef EBB_UPD_MINB_D
#define EBB_UPD_MINB_D 4
#endif
#ifndef EBB_UPD_MINB_W
#define EBB_UPD_MINB_W 4
#endif
