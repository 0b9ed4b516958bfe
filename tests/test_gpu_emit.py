"""Device-side emission (sphmp_set_device_emitter) against the host path of the
reference's EmitParticles (sphmp_emit_disk + sphmp_emit_aos before the step, the
EmitUpdateCUDA route). Both are integer-exact in what they emit and the step
is deterministic, so the tolerance is zero: every record and every sort array
must be identical after several steps with emissions, and the count must stop
at the capacity with SPHMP_ERR_CAPACITY reported."""
import numpy as np
import pytest

import sphmp
from helpers import bits_equal, download_state
from sphmp import abi, scenes

pytestmark = pytest.mark.gpu

EMITTER = dict(position=(0.09, 0.16, 0.08), direction=(0.0, -1.0, 0.0), speed=0.5, radius=0.03, spacing=0.01)
SEED = 11


def _scene(spare):
    sc = scenes.small_block(seed=61, n=(10, 8, 9), nphase=2, eos=abi.EOS_TAIT, velocity_scale=0.2,
                            box=(0.2, 0.24, 0.2))
    sc.params.maxNum = sc.n + spare
    disp, calc = sphmp.record_arrays(sc.n + spare)
    disp[:sc.n] = sc.disp[:sc.n]
    calc[:sc.n] = sc.calc[:sc.n]
    return sc, disp, calc


def _host_emit(ctx, p, disp, calc, frame, layers, phase):
    n0 = ctx.n
    n1 = sphmp.emit_disk(p, disp, calc, n0, EMITTER["position"], EMITTER["direction"], EMITTER["speed"],
                         EMITTER["radius"], EMITTER["spacing"], layers=layers, phase=phase, frame=frame,
                         jitter=1.0, seed=SEED + frame)
    ctx.emit_aos(disp[n0:n1], calc[n0:n1], n0, n1)


@pytest.mark.parametrize("use_graph", [True, False], ids=["graph", "eager"])
def test_device_emission_matches_host_emission(built, use_graph):
    sc, disp, calc = _scene(spare=2000)
    p = sc.params
    interval, layers, phase, steps = 3, 2, 1, 8
    dev = sphmp.Context(p)
    dev.upload_aos(disp[:sc.n], calc[:sc.n])
    dev.before_first_step()
    dev.set_device_emitter(**EMITTER, layers=layers, phase=phase, interval=interval, jitter=1.0, seed=SEED)
    dev.step(steps, abi.SCHEDULE_FUSED, use_graph=use_graph)
    dev.sync()
    host = sphmp.Context(p)
    host.upload_aos(disp[:sc.n], calc[:sc.n])
    host.before_first_step()
    for f in range(steps):
        if f % interval == 0:
            _host_emit(host, p, disp, calc, f, layers, phase)
        host.step(1, abi.SCHEDULE_FUSED, use_graph=use_graph)
    host.sync()
    assert dev.n == host.n and dev.n > sc.n + 3 * 40
    assert dev.device_errors() == 0 and host.device_errors() == 0
    a, b = download_state(dev), download_state(host)
    for k in a:
        assert bits_equal(a[k], b[k]), k
    da, ca = dev.download_aos()
    db, cb = host.download_aos()
    assert da.tobytes() == db.tobytes() and ca.tobytes() == cb.tobytes()
    dev.close()
    host.close()


def test_device_emission_stops_at_capacity(built):
    sc, disp, calc = _scene(spare=60)
    dev = sphmp.Context(sc.params)
    dev.upload_aos(disp[:sc.n], calc[:sc.n])
    dev.before_first_step()
    dev.set_device_emitter(**EMITTER, layers=2, phase=0, interval=1, seed=SEED)
    dev.step(3, abi.SCHEDULE_FUSED, use_graph=True)
    assert dev.device_errors() & (1 << abi.ERR_CAPACITY)  # read (and cleared) before sync would raise it
    dev.sync()
    assert dev.n == sc.n + 60
    # the emitted particles are fluid records of phase 0 with their own slots as bornid
    d, c = dev.download_aos()
    born = np.sort(c["bornid"])
    assert np.array_equal(born, np.arange(sc.n + 60))
    new = c["bornid"] >= sc.n
    assert np.all(d["type"][new] == abi.TYPE_FLUID)
    assert np.all(c["mass"][new] == np.float32(sc.params.massArr[0]))
    # off again: the count stays, steps go on
    dev.set_device_emitter(**EMITTER, interval=0)
    dev.step(2, abi.SCHEDULE_FUSED, use_graph=True)
    dev.sync()
    assert dev.n == sc.n + 60 and dev.device_errors() == 0
    dev.close()


def test_device_emitter_rejects_bad_settings(built):
    sc, disp, calc = _scene(spare=10)
    dev = sphmp.Context(sc.params)
    dev.upload_aos(disp[:sc.n], calc[:sc.n])
    bad = [dict(EMITTER, spacing=0.0), dict(EMITTER, radius=-1.0), dict(EMITTER, radius=100.0, spacing=1e-4)]
    for e in bad:
        with pytest.raises(sphmp.SphmpError) as err:
            dev.set_device_emitter(**e, interval=3)
        assert err.value.status == abi.ERR_INVALID_ARG
    with pytest.raises(sphmp.SphmpError) as err:
        dev.set_device_emitter(**EMITTER, phase=5, interval=3)
    assert err.value.status == abi.ERR_INVALID_ARG
    dev.close()

