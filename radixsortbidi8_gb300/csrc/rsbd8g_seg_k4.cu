// rsbd8g_seg_k4.cu - the batched (segmented) sort for 32-bit keys.
#include "rsbd8g_seglaunch.cuh"

RSBD8G_DEFINE_SEG_LAUNCH(launch_segmented_k4, uint32_t)
