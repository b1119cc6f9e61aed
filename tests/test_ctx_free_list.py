"""Every device buffer of a context is released by yg_destroy.

A static check of the sources: each device-pointer field of struct yg_ctx
(yg_internal.cuh) is named in yg_destroy's free list (yg_capi.cu).  A field
left out would stay allocated in the library's memory pool after the context
is destroyed (yg_destroy also frees whatever allocation is left over, so this
guards the explicit list)."""
import os
import re

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), 'yaff_gb300', 'csrc')


def test_destroy_names_every_device_field():
    src = open(os.path.join(CSRC, 'yg_internal.cuh')).read()
    body = re.search(r'struct yg_ctx\s*\{(.*?)\n\};', src, re.S).group(1)
    fields = set(re.findall(r'\*\s*(d_\w+)\s*(?:=|;|\[)', body))
    cap = open(os.path.join(CSRC, 'yg_capi.cu')).read()
    d = cap[cap.index('int yg_destroy'):cap.index('int yg_set_precision')]
    freed = set(re.findall(r'c->(d_\w+)', d))
    assert fields, 'no device fields found'
    assert not (fields - freed), sorted(fields - freed)
