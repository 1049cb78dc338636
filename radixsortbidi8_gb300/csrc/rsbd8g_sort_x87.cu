// rsbd8g_sort_x87.cu - the sort kernels and launch sequence for x87 extended precision keys in 16-byte storage (10 digits).
#include "rsbd8g_launch.cuh"

RSBD8G_DEFINE_LAUNCH(launch_sort_x87, rsbd8g::KeyX87)
