// rsbd8g_sort_k8.cu - the sort kernels and launch sequence for 64-bit keys.
#include "rsbd8g_launch.cuh"

RSBD8G_DEFINE_LAUNCH(launch_sort_k8, uint64_t)
