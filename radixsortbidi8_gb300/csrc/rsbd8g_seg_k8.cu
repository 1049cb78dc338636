// rsbd8g_seg_k8.cu - the batched (segmented) sort for 64-bit keys.
#include "rsbd8g_seglaunch.cuh"

RSBD8G_DEFINE_SEG_LAUNCH(launch_segmented_k8, uint64_t)
