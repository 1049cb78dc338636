// Host-side checks of rsbd8g::sort_array, the lookup by which the scatter and copy kernels turn the
// array indices of the control block into addresses: a valid index gives its array, kArrNone gives
// null, and an index that names no array (out of range, or an array the call does not have) gives
// the fallback array and sets the fault flag.  Built with nvcc, run on the host (no GPU needed).
#include <cstdio>

#include "rsbd8g_device.cuh"

using namespace rsbd8g;

static int failures = 0;
static void check(bool ok, const char *what) {
    if (!ok) {
        std::printf("FAIL: %s\n", what);
        ++failures;
    }
}

int main() {
    int in = 0, out = 0, buf = 0, ka = 0;
    SortArrays a{};
    a.p[kArrIn] = &in;
    a.p[kArrOut] = &out;
    a.p[kArrBuf] = &buf;
    a.p[kArrKeysA] = &ka;
    a.p[kArrKeysB] = nullptr;          // a direct sort's second key array: absent
    bool bad = false;
    check(sort_array(a, kArrIn, kArrBuf, &bad) == &in && !bad, "input");
    check(sort_array(a, kArrOut, kArrBuf, &bad) == &out && !bad, "output");
    check(sort_array(a, kArrBuf, kArrIn, &bad) == &buf && !bad, "buffer");
    check(sort_array(a, kArrKeysA, kArrIn, &bad) == &ka && !bad, "keys A");
    check(sort_array(a, kArrNone, kArrIn, &bad) == nullptr && !bad, "none");
    bad = false;
    check(sort_array(a, kArrKeysB, kArrBuf, &bad) == &buf && bad, "an absent array falls back and is flagged");
    for (uint32_t sel : {5u, 6u, 77u, 0xFEu, 0x100u, 0xFFFFFFFFu}) {
        bad = false;
        check(sort_array(a, sel, kArrIn, &bad) == &in && bad, "an index that names no array falls back and is flagged");
    }
    static_assert(sizeof(Control) <= 1024, "control block slot");
    static_assert(sizeof(PassPlan) == 32, "pass plan layout");
    if (failures == 0) std::printf("ok\n");
    return failures == 0 ? 0 : 1;
}
