"""Error paths under injected allocation failures (sc_test_fail_allocations).

Every entry point that allocates device workspace is made to fail at each of
its allocations in turn.  Each failure must come back as SC_ERR_OOM with a
message.  The same call on the same object, with allocations allowed again,
must then succeed and give the result of an object that never failed.  A
second pass fails one allocation at a time on a single object, so that each
retry starts from a partly allocated workspace.  No device memory is
actually exhausted: the hook fails allocations before the runtime is called.

Also: a batch graph is recaptured when a member mesh is refitted between
calls (its geometry is a kernel argument captured by value)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SC_ERR_OOM = 3
MAX_ALLOCS = 64


@pytest.fixture
def inject(sc, cuda):
    lib = sc.load()
    yield lambda k: lib.sc_test_fail_allocations(k)
    lib.sc_test_fail_allocations(-1)


def _bunch(torch, n, seed, spread=1e-3, dtype=None):
    dtype = dtype or torch.float64
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((3, n)) * spread
    a[2] = np.abs(a[2]) * 3 + 1e-4  # above the cathode plane z = 0
    dev = [torch.from_numpy(v).to("cuda", dtype).contiguous() for v in a]
    dev.append(torch.full((n,), 1e-9 / n, dtype=dtype, device="cuda"))
    return dev


def _close(got, want, rtol):
    for a, b in zip(got, want):
        scale = float(b.abs().max())
        assert scale > 0
        assert float((a - b).abs().max()) <= rtol * scale


def _call(sc, inject, k, op, obj):
    """op(obj) with allocations failing after k successes; returns (out, failed)."""
    inject(k)
    try:
        return op(obj), False
    except sc.SpaceChargeError as e:
        assert e.code == SC_ERR_OOM, (k, e.code, str(e))
        assert "error" in str(e).lower()
        return None, True
    finally:
        inject(-1)


def _drive(sc, torch, inject, make, op, want, rtol):
    """Fail at allocation k = 0, 1, ... of op on a fresh object each time,
    then retry on the same object; then fail one allocation at a time on a
    single object until op goes through.  Returns op's allocation count."""
    needed = None
    for k in range(MAX_ALLOCS):
        obj = make()
        out, failed = _call(sc, inject, k, op, obj)
        if failed:
            out = op(obj)
        torch.cuda.synchronize()
        _close(out, want, rtol)
        if not failed:
            needed = k
            break
    assert needed is not None, f"op still failing after {MAX_ALLOCS} allocations"
    obj = make()
    for _ in range(needed + 1):
        out, failed = _call(sc, inject, 1, op, obj)
        if not failed:
            break
    else:
        out = op(obj)
    torch.cuda.synchronize()
    _close(out, want, rtol)
    return needed


def _kick_case(sc, torch, inject, precision, mode, at_cathode, rtol, n=20_000, grid=(16, 16, 16)):
    dev = _bunch(torch, n, 7)

    def make():
        m = sc.Mesh3D(grid, dev[0], dev[1], dev[2], precision=precision)
        if mode:
            m.set_kick_mode(mode)
        return m

    ref = make()
    ref.set_kick_graph(False)
    want = [t.clone() for t in sc.kick(ref, *dev, at_cathode=at_cathode)]

    def op(m):
        return [t.clone() for t in sc.kick(m, *dev, at_cathode=at_cathode)]

    return _drive(sc, torch, inject, make, op, want, rtol)


@pytest.mark.parametrize("precision,mode,at_cathode,rtol", [
    ("mixed", None, True, 1e-5),
    ("mixed", "sorted", False, 1e-5),
    ("mixed", "deterministic", False, 1e-5),
    ("mixed", "tiled", False, 1e-5),
    ("fp64", None, False, 1e-10),
    ("plain64", None, True, 1e-10),
])
def test_kick_survives_each_allocation_failure(sc, cuda, inject, precision, mode, at_cathode, rtol):
    needed = _kick_case(sc, cuda, inject, precision, mode, at_cathode, rtol)
    assert needed >= 1  # the kick allocates its workspace on first use


def test_mesh_create_reports_oom(sc, cuda, inject):
    dev = _bunch(cuda, 1000, 1)
    for k in range(3):  # rho, efield, the out-of-range counter
        inject(k)
        try:
            with pytest.raises(sc.SpaceChargeError) as ei:
                sc.Mesh3D((8, 8, 8), dev[0], dev[1], dev[2], precision="mixed")
        finally:
            inject(-1)
        assert ei.value.code == SC_ERR_OOM
    sc.Mesh3D((8, 8, 8), dev[0], dev[1], dev[2], precision="mixed")


def test_host_kick_survives_each_allocation_failure(sc, cuda, inject):
    torch = cuda
    dev = _bunch(torch, 200_000, 3)
    host = [t.cpu() for t in dev]

    def make():
        return sc.Mesh3D((16, 16, 16), dev[0], dev[1], dev[2], precision="mixed")

    ref = make()
    ref.set_kick_graph(False)
    want = [t.clone().cpu() for t in sc.kick(ref, *dev)]

    def op(m):
        return [t.clone() for t in sc.kick_host(m, *host)]

    _drive(sc, torch, inject, make, op, want, 1e-5)


def test_adjoint_survives_each_allocation_failure(sc, cuda, inject):
    torch = cuda
    dev = _bunch(torch, 20_000, 5)
    # zero-mean upstream gradients, as in the adjoint's own tests: a coherent
    # one (all ones) makes the position gradient a small difference of large
    # terms, at the FP32 pipeline's rounding level
    g = torch.from_numpy(np.random.default_rng(6).standard_normal((3, 20_000))).cuda()

    def make():
        return sc.Mesh3D((16, 16, 16), dev[0], dev[1], dev[2], precision="mixed")

    want = [t.clone() for t in sc.kick_adjoint(make(), *dev, *g)]

    def op(m):
        return [t.clone() for t in sc.kick_adjoint(m, *dev, *g)]

    _drive(sc, torch, inject, make, op, want, 1e-4)


def test_track_survives_each_allocation_failure(sc, cuda, inject):
    torch = cuda
    dev = _bunch(torch, 20_000, 9)
    u = [torch.zeros_like(dev[0]), torch.zeros_like(dev[0]), torch.full_like(dev[0], 10.0)]

    def make():
        return sc.Mesh3D((16, 16, 16), dev[0], dev[1], dev[2], precision="fp64", gamma=float(np.sqrt(101.0)))

    def op(m):
        st = [t.clone() for t in dev[:3] + u]
        sc.track(m, *st, dev[3], dt=1e-12, qm=-1.75882001076e11, steps=2, refit=True)
        return st

    want = op(make())
    _drive(sc, torch, inject, make, op, want, 1e-12)


def test_potential_survives_each_allocation_failure(sc, cuda, inject):
    torch = cuda
    dev = _bunch(torch, 20_000, 11)

    def make():
        m = sc.Mesh3D((16, 16, 16), dev[0], dev[1], dev[2], precision="mixed")
        sc.deposit(m, *dev, mode="deterministic")
        return m

    want = [sc.solve_potential(make(), at_cathode=True).clone()]

    def op(m):
        return [sc.solve_potential(m, at_cathode=True).clone()]

    _drive(sc, torch, inject, make, op, want, 1e-10)


def test_batch_survives_each_allocation_failure(sc, cuda, inject):
    torch = cuda
    bunches = [_bunch(torch, n, 20 + i) for i, n in enumerate((15_000, 40_000))]

    def make():
        ms = [sc.Mesh3D(g, b[0], b[1], b[2], precision="mixed") for g, b in zip(((16, 16, 16), (8, 16, 32)), bunches)]
        return sc.Batch(ms, nstreams=2)

    want = []
    for g, b in zip(((16, 16, 16), (8, 16, 32)), bunches):
        r = sc.Mesh3D(g, b[0], b[1], b[2], precision="mixed")
        r.set_kick_graph(False)
        want.extend(t.clone() for t in sc.kick(r, *b))

    def op(batch):
        outs = batch.kick(*[[b[k] for b in bunches] for k in range(4)])
        return [t.clone() for o in outs for t in o]

    _drive(sc, torch, inject, make, op, want, 1e-5)


def test_batch_graph_follows_member_refit(sc, cuda):
    """A member mesh refitted by sc_track between two batch kicks: the second
    kick uses the new geometry, as an eager kick on that geometry does."""
    torch = cuda
    b0, b1 = _bunch(torch, 30_000, 31), _bunch(torch, 30_000, 32)
    wide = _bunch(torch, 30_000, 33, spread=2.5e-3)
    m0 = sc.Mesh3D((16, 16, 16), b0[0], b0[1], b0[2], precision="mixed")
    m1 = sc.Mesh3D((16, 16, 16), b1[0], b1[1], b1[2], precision="mixed")
    batch = sc.Batch([m0, m1], nstreams=2)
    args = [[b0[k], b1[k]] for k in range(4)]
    first = [t.clone() for t in batch.kick(*args)[0]]
    replay = [t.clone() for t in batch.kick(*args)[0]]
    _close(replay, first, 1e-5)
    # refit m0 to the wider bunch without moving it (dt = 0)
    st = [t.clone() for t in wide[:3]] + [torch.zeros_like(wide[0]) for _ in range(3)]
    sc.track(m0, *st, wide[3], dt=0.0, qm=0.0, steps=1, refit=True)
    after = [t.clone() for t in batch.kick(*args)[0]]
    ref = sc.Mesh3D((16, 16, 16), wide[0], wide[1], wide[2], precision="mixed")
    ref.set_kick_graph(False)
    want = [t.clone() for t in sc.kick(ref, *b0)]
    _close(after, want, 1e-5)
    assert float((after[2] - first[2]).abs().max()) > 1e-3 * float(first[2].abs().max())
