// Generated by ebbcfd_gb300/autotune.py on the default-size plate workload: device time per
// launch of each kernel of both precision forms for each (threads per block) x (minimum
// resident blocks per SM requested through __launch_bounds__; 1 = the compiler's
// register choice), best of three rounds of CUDA-event timing; fastest kept.
// split k_cell: 64x12 136.4 us, 64x16 146.4 us, 128x6 137.5 us, 128x8 146.4 us, 128x10 167.3 us, 256x3 138.4 us, 256x4 149.0 us
// split k_flux: 64x16 133.9 us, 64x20 124.6 us, 128x8 135.2 us, 128x10 125.6 us, 128x12 115.6 us, 256x4 149.4 us, 256x6 119.2 us
// split k_update: 256x4 135.4 us, 256x6 142.0 us, 256x8 150.1 us, 512x2 151.2 us, 512x3 148.0 us, 512x4 155.9 us
// fp64 k_cell: 64x8 3038.0 us, 64x10 3026.3 us, 128x1 3045.0 us, 128x5 3026.3 us, 128x6 3029.3 us, 256x2 3050.1 us, 256x3 3040.5 us
// fp64 k_flux: 64x6 5416.3 us, 64x8 5417.5 us, 128x1 5417.8 us, 128x4 5417.7 us, 128x5 5467.3 us, 256x1 5436.3 us, 256x2 5436.3 us
// fp64 k_update: 256x1 661.7 us, 256x2 662.5 us, 256x3 566.2 us, 256x4 567.0 us, 512x1 761.3 us, 512x2 603.9 us
// update block size 256 (summed best update times: 256: 701.6 us, 512: 751.9 us)
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
#define EBB_CELL_TB_D 64
#endif
#ifndef EBB_CELL_MINB_D
#define EBB_CELL_MINB_D 10
#endif
#ifndef EBB_FLUX_TB_D
#define EBB_FLUX_TB_D 64
#endif
#ifndef EBB_FLUX_MINB_D
#define EBB_FLUX_MINB_D 6
#endif
#ifndef EBB_UPD_TB
#define EBB_UPD_TB 256
#endif
#ifndef EBB_UPD_MINB_F
#define EBB_UPD_MINB_F 4
#endif
#ifndef EBB_UPD_MINB_D
#define EBB_UPD_MINB_D 3
#endif
