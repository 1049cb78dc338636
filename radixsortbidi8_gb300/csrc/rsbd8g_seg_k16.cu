// rsbd8g_seg_k16.cu - the batched (segmented) sort for 16-byte keys: 128-bit integers and 128-bit float words.
#include "rsbd8g_seglaunch.cuh"

RSBD8G_DEFINE_SEG_LAUNCH(launch_segmented_k16, rsbd8g::KeyU128)
