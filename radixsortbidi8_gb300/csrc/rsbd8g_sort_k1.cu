// rsbd8g_sort_k1.cu - the sort kernels and launch sequence for 8-bit keys.
#include "rsbd8g_launch.cuh"

RSBD8G_DEFINE_LAUNCH(launch_sort_k1, uint8_t)
