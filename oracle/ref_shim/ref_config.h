/* Values for the configuration macros that fwi_2d.c's fwi_init/rwi_init use
 * but that are defined nowhere in the reference (they lived in a missing
 * file).  The oracle never calls fwi_init/rwi_init; these only let the
 * translation unit compile so its propagator kernels can be linked. */
#define NT_MEM 100
#define FREE_SURFACE 1
#define NR 8
#define DR 10.0
#define DAT_JUMP 2
#define DAT_RECT_X 1
#define DAT_RECT_T 1
#define DAT_SM_TIMES 1
#define OFFSET0 0.0
#define OFFSET1 1.0e9
#define FBT_UP 0
#define FBT_DOWN 0
#define MSF_SCALE 1.0
#define TUNE_BTRY 0.0
#define WAV_SCALE 1.0
#define WAVELET_est "%swavelet_%d_%d.bin"
#define STEP 1
#define G_END_T 1.0
#define G_START_T 0.0
#define G_SCALE 1.0
#define G_PERC 0.0
#define G_JUMP 1
#define G_SM_RECTX1 1
#define G_SM_RECTZ1 1
#define G_SM_TIMES1 1
#define G_SM_RECTX2 1
#define G_SM_RECTZ2 1
#define G_SM_TIMES2 1
#define INIT_MDL_0 "%sinput/m0.bin"
#define INIT_MDL_1 "%sinput/m1.bin"
