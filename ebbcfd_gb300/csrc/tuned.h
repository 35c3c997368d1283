// Generated by ebbcfd_gb300/autotune.py on the default-size plate workload: device time per
// launch of each kernel of the three precision forms for each (threads per block) x (minimum
// resident blocks per SM requested through __launch_bounds__; 1 = the compiler's
// register choice), best of three rounds of CUDA-event timing; fastest kept.
// split k_cell: 64x12 137.1 us, 64x16 146.6 us, 128x6 138.0 us, 128x8 146.7 us, 128x10 167.5 us, 256x3 139.8 us, 256x4 149.2 us
// split k_flux: 64x16 133.7 us, 64x20 124.0 us, 128x8 135.0 us, 128x10 124.9 us, 128x12 115.8 us, 256x4 149.2 us, 256x6 119.7 us
// split k_update: 256x4 135.6 us, 256x6 137.6 us, 256x8 150.3 us, 512x2 140.3 us, 512x3 143.8 us, 512x4 156.8 us
// fp64 k_cell: 64x8 2822.5 us, 64x10 2808.5 us, 128x1 2822.5 us, 128x5 2807.9 us, 128x6 2807.2 us, 256x2 2840.5 us, 256x3 2813.9 us
// fp64 k_flux: 64x6 5177.3 us, 64x8 5175.1 us, 128x1 5179.4 us, 128x4 5176.9 us, 128x5 5251.0 us, 256x1 5194.2 us, 256x2 5195.5 us
// fp64 k_update: 256x1 662.5 us, 256x2 663.3 us, 256x3 567.2 us, 256x4 567.1 us, 512x1 762.1 us, 512x2 605.3 us
// df k_cell: 64x4 1035.3 us, 64x6 1026.0 us, 128x1 1018.2 us, 128x2 1018.4 us, 128x3 1017.0 us, 256x1 1355.9 us, 256x2 824.7 us
// df k_flux: 64x4 761.0 us, 64x6 761.3 us, 128x1 756.1 us, 128x2 754.0 us, 128x3 755.3 us, 256x1 757.9 us, 256x2 758.3 us
// df k_update: 256x1 409.5 us, 256x2 409.6 us, 256x3 293.6 us, 256x4 256.0 us, 512x1 465.2 us, 512x2 289.0 us
// split_inv k_cell: 64x12 30.9 us, 64x16 27.4 us, 128x6 31.9 us, 128x8 27.8 us, 128x10 32.5 us, 256x3 32.8 us, 256x4 27.8 us
// split_inv k_flux: 64x16 27.0 us, 64x20 26.9 us, 128x8 23.4 us, 128x10 22.3 us, 128x12 20.3 us, 256x4 25.4 us, 256x6 20.9 us
// split_inv k_update: 256x4 32.3 us, 256x6 30.0 us, 256x8 28.9 us, 512x2 35.3 us, 512x3 30.6 us, 512x4 29.3 us
// update block size 256 (summed best update times: 256: 987.6 us, 512: 1063.9 us)
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
#define EBB_FLUX_MINB_D 8
#endif
#ifndef EBB_CELL_TB_W
#define EBB_CELL_TB_W 256
#endif
#ifndef EBB_CELL_MINB_W
#define EBB_CELL_MINB_W 2
#endif
#ifndef EBB_FLUX_TB_W
#define EBB_FLUX_TB_W 128
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
#ifndef EBB_CELL_TB_FI
#define EBB_CELL_TB_FI 64
#endif
#ifndef EBB_CELL_MINB_FI
#define EBB_CELL_MINB_FI 16
#endif
#ifndef EBB_FLUX_TB_FI
#define EBB_FLUX_TB_FI 128
#endif
#ifndef EBB_FLUX_MINB_FI
#define EBB_FLUX_MINB_FI 12
#endif
#ifndef EBB_UPD_MINB_FI
#define EBB_UPD_MINB_FI 8
#endif
