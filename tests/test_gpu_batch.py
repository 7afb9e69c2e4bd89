"""Batched ensemble (asam_batch_*): members of different sizes, orography and
wind advanced together give exactly what each member gives alone."""
import numpy as np
import pytest

from tests import cases

pytestmark = pytest.mark.gpu

MEMBERS = ["hill_24x20x16", "hill_odd_13x7x9_reverse", "flat_walls_9x6x5", "column_1x1x12", "slab_1x9x6",
           "bubble_12x10x8"]


@pytest.fixture(scope="module")
def asam(built_lib):
    import asam_gb300

    return asam_gb300


def _blocks(asam, **kw):
    out = []
    for name in MEMBERS:
        geo, vel, st = cases.get(name)
        b = asam.TransportBlock(geo, ncomp=st.c.shape[0], rho_pos=st.rho_pos, method="RosRK3", **kw)
        b.set_velocity(*vel)
        out.append((b, st))
    return out


@pytest.mark.parametrize("precision", ["fp64", "fp32_refined"])
@pytest.mark.parametrize("nthreads", [1, 0])
def test_batch_matches_members_alone(asam, precision, nthreads):
    kw = dict(bicgstab_tol=1e-10, precision=precision)
    dts = [2.0, 3.0, 1.5, 2.5, 2.0, 4.0]
    alone = []
    for (b, st), dt in zip(_blocks(asam, **kw), dts):
        c = st.c.copy()
        its = [b.Ros3MetC(c, dt)[0] for _ in range(3)]
        alone.append((c, its))
        b.close()
    members = _blocks(asam, **kw)
    states = [st.c.copy() for _, st in members]
    with asam.Batch([b for b, _ in members], nthreads=nthreads) as batch:
        its, status = batch.ros_step(states, dts, nsteps=3)
    for b, _ in members:
        b.close()
    # statuses carry the members' own BiCGStab outcomes (the one-column member
    # reaches the iteration limit alone too); the iteration sentinels must match
    assert all(int(x) in (0, 1) for x in status), status
    for m, (c_ref, its_ref) in enumerate(alone):
        assert np.array_equal(states[m], c_ref), MEMBERS[m]
        assert [list(map(int, s)) for s in its[m]] == its_ref, MEMBERS[m]


@pytest.mark.parametrize("precision", ["fp64", "fp32_refined"])
def test_batch_graph_matches_members_alone(asam, precision):
    """One-graph mode: the whole 3-step run of every member as one CUDA graph
    launch (refined members: the FP64 refinement and the FP32 BiCGStab as
    nested WHILE nodes) gives bitwise the states and iteration counts of each
    member run alone; a second call replays the graph."""
    import torch

    kw = dict(bicgstab_tol=1e-10, precision=precision)
    dts = [2.0, 3.0, 1.5, 2.5, 2.0, 4.0]
    alone = []
    for (b, st), dt in zip(_blocks(asam, **kw), dts):
        c = st.c.copy()
        its = [b.Ros3MetC(c, dt)[0] for _ in range(6)]
        alone.append((c, its))
        b.close()
    members = _blocks(asam, **kw)
    dev = [torch.from_numpy(st.c.reshape(-1).copy()).cuda() for _, st in members]
    torch.cuda.synchronize()
    host0 = members[0][1].c.copy()
    with asam.Batch([b for b, _ in members]) as batch:
        batch.set_graph(True)
        its1, status1 = batch.ros_step([t.data_ptr() for t in dev], dts, nsteps=3)
        its2, status2 = batch.ros_step([t.data_ptr() for t in dev], dts, nsteps=3)  # replay
        batch.set_graph(False)
    torch.cuda.synchronize()
    for b, _ in members:
        b.close()
    assert all(int(x) in (0, 1) for x in status1) and all(int(x) in (0, 1) for x in status2)
    for m, (c_ref, its_ref) in enumerate(alone):
        got = dev[m].cpu().numpy().reshape(c_ref.shape)
        assert np.array_equal(got, c_ref), MEMBERS[m]
        its = [list(map(int, s)) for s in its1[m]] + [list(map(int, s)) for s in its2[m]]
        assert its == its_ref, MEMBERS[m]
    assert np.array_equal(host0, members[0][1].c)


def test_batch_graph_sees_member_changes(asam):
    """A member's wall rule changed after the ensemble graph was recorded
    (flat_walls_9x6x5: ZeroValue on every wall for every component but the
    density -- negating the density too would leave every halo's mixing
    ratio, and so the fluxes, as they were) makes the next call record the
    graph again: the states equal the members run alone with the old rule
    for the first call and the new one after."""
    import torch

    kw = dict(bicgstab_tol=1e-10)
    dts = [2.0, 3.0, 1.5, 2.5, 2.0, 4.0]
    m_walls = MEMBERS.index("flat_walls_9x6x5")
    st_walls = cases.get("flat_walls_9x6x5")[2]
    zero_value = np.full((st_walls.c.shape[0], 6), 2, np.int32)
    zero_value[st_walls.rho_pos] = 1
    alone = []
    for m, ((b, st), dt) in enumerate(zip(_blocks(asam, **kw), dts)):
        c = st.c.copy()
        b.Ros3MetC(c, dt)
        if m == m_walls:
            kept = c.copy()
            b.Ros3MetC(kept, dt)  # the old rule: what a stale graph would give
            b.set_boundary(zero_value)
        b.Ros3MetC(c, dt)
        if m == m_walls:
            assert not np.array_equal(c, kept)
        alone.append(c)
        b.close()
    members = _blocks(asam, **kw)
    dev = [torch.from_numpy(st.c.reshape(-1).copy()).cuda() for _, st in members]
    torch.cuda.synchronize()
    with asam.Batch([b for b, _ in members]) as batch:
        batch.set_graph(True)
        batch.ros_step([t.data_ptr() for t in dev], dts, nsteps=1)
        members[m_walls][0].set_boundary(zero_value)
        batch.ros_step([t.data_ptr() for t in dev], dts, nsteps=1)
    torch.cuda.synchronize()
    for b, _ in members:
        b.close()
    for m, c_ref in enumerate(alone):
        assert np.array_equal(dev[m].cpu().numpy().reshape(c_ref.shape), c_ref), MEMBERS[m]


def test_batch_device_states(asam):
    import torch

    members = _blocks(asam, bicgstab_tol=1e-10)
    host = [st.c.copy() for _, st in members]
    dev = [torch.from_numpy(st.c.reshape(-1).copy()).cuda() for _, st in members]
    torch.cuda.synchronize()  # the members' streams do not wait for torch's
    with asam.Batch([b for b, _ in members]) as batch:
        batch.ros_step(host, 2.0, nsteps=2)
        batch.ros_step([t.data_ptr() for t in dev], 2.0, nsteps=2)
    torch.cuda.synchronize()
    for h, d in zip(host, dev):
        assert np.array_equal(h.reshape(-1), d.cpu().numpy())
    for b, _ in members:
        b.close()


def test_batch_rejects_bad_arguments(asam):
    members = _blocks(asam)
    b0 = members[0][0]
    with pytest.raises(Exception):
        asam.Batch([b0, b0])  # one context twice
    with asam.Batch([b for b, _ in members]) as batch:
        with pytest.raises(ValueError):
            batch.ros_step([members[0][1].c.copy()], 2.0)
    for b, _ in members:
        b.close()
