// rsbd8g_seg_k2.cu - the batched (segmented) sort for 16-bit keys.
#include "rsbd8g_seglaunch.cuh"

RSBD8G_DEFINE_SEG_LAUNCH(launch_segmented_k2, uint16_t)
