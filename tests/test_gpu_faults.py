"""Failure paths on the GPU, exercised without faulting it.

Every device-side wait of the trace (the mbarrier wait for the bulk copy of the object table
into shared memory, lg_trace.cu stage_objects) is bounded.  A context created with
lg_device_opts.wait_polls < 0 gives up on the first poll: the kernel records the timeout in
the device error flags, still waits (bounded) for its own copy to land, and returns, so the
host reports LG_ERR_TIMEOUT and the GPU stays usable.  Nothing here traps, faults or hangs.
"""
import pytest

from light_garden_gb300 import abi, workloads as W

pytestmark = pytest.mark.gpu


def test_object_table_wait_gives_up_with_timeout(gpu):
    from light_garden_gb300.runtime import Context

    pk = W.plain_small(accum=abi.LG_ACCUM_FIXED64, num_rays=256).packed()
    with Context(wait_polls=-1) as ctx:
        ctx.upload(pk)
        with pytest.raises(abi.LgError) as e:
            ctx.trace()
        assert e.value.status == abi.LG_ERR_TIMEOUT
        # the whole frame path reports it as well
        with pytest.raises(abi.LgError) as e:
            ctx.render()
        assert e.value.status == abi.LG_ERR_TIMEOUT
    # the device is still usable: a context with the default limit traces the same scene
    with Context() as ctx:
        ctx.upload(pk)
        st = ctx.trace()
        assert st["segments"] > 256
