// rsbd8g_seg_k1.cu - the batched (segmented) sort for 8-bit keys.
#include "rsbd8g_seglaunch.cuh"

RSBD8G_DEFINE_SEG_LAUNCH(launch_segmented_k1, uint8_t)
