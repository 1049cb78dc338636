// rsbd8g_sort_k2.cu - the sort kernels and launch sequence for 16-bit keys.
#include "rsbd8g_launch.cuh"

RSBD8G_DEFINE_LAUNCH(launch_sort_k2, uint16_t)
