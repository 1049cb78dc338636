"""rsbd8 on GB300: a device-resident stable LSD radix sort with the rsbd8 API.

The sort runs as hand-written sm_103a kernels in ``librsbd8g.so`` behind the C ABI
of ``include/rsbd8g.h``; this package is the Python host mirror of that API.
"""
from .api import (  # noqa: F401
    DIRECTIONS, MODES, RSBD8GError, Desc, key_kind, lib, make_desc, radixsort, radixsortcopy,
    radixsortcopy_member, radixsortcopynoalloc, radixsortcopynoalloc_member, radixsort_member,
    radixsortnoalloc, scratch_bytes, scratch_status,
)

__all__ = [
    "DIRECTIONS", "MODES", "RSBD8GError", "Desc", "key_kind", "lib", "make_desc", "radixsort",
    "radixsortcopy", "radixsortcopy_member", "radixsortcopynoalloc", "radixsortcopynoalloc_member",
    "radixsort_member", "radixsortnoalloc", "scratch_bytes", "scratch_status",
]
