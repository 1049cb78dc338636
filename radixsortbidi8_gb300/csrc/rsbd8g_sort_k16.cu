// rsbd8g_sort_k16.cu - the sort kernels and launch sequence for 16-byte keys: 128-bit integers and 128-bit float words.
#include "rsbd8g_launch.cuh"

RSBD8G_DEFINE_LAUNCH(launch_sort_k16, rsbd8g::KeyU128)
