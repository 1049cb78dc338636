// rsbd8g_sort_k4.cu - the sort kernels and launch sequence for 32-bit keys.
#include "rsbd8g_launch.cuh"

RSBD8G_DEFINE_LAUNCH(launch_sort_k4, uint32_t)
