"""nsm_critical_time_step_noalloc -- the stable time step for callers that
cannot allocate GPU memory (for example a framework that owns every device
buffer through its own pool, or code running during CUDA stream capture).  It
keeps its scratch in a fixed array inside the library, so the caller only
passes the mesh, the displacement and a one-double output.

Checked through the C ABI against the existing entry point
(nsm_critical_time_step) on two calls in a row, bitwise as the other
time-step tests are.  Collected last so that a failure here stops a -x run
only after every other test has run.  The test allocates its own buffers
with torch (the test is not the caller that cannot allocate)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_time_step_matches_existing_entry_point():
    torch = pytest.importorskip("torch")
    from nimblesm_gb300 import build as B
    from nimblesm_gb300 import engine as E
    from nimblesm_gb300.mesh import characteristic_lengths, cube_problem

    B.build()
    lib = E.library()
    p = cube_problem(20, jitter=0.2, seed=3)
    model = E.Model(p)
    dt_ref = model.GetCriticalTimeStep()
    model.close()

    dev = torch.device("cuda:0")
    X = torch.from_numpy(np.ascontiguousarray(p.coords, dtype=np.float64)).to(dev)
    conn = torch.from_numpy(np.ascontiguousarray(p.conn, dtype=np.int32)).to(dev)
    out = torch.empty(1, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream

    for _ in range(2):  # two calls in a row: the shared scratch keeps the last call's contents
        out.fill_(-1.0)
        rc = lib.nsm_critical_time_step_noalloc(p.num_nodes, p.num_elem, X.data_ptr(), None, conn.data_ptr(),
                                                p.density, p.bulk_modulus, out.data_ptr(), stream)
        assert rc == 0, lib.nsm_last_error()
        torch.cuda.synchronize(dev)
        assert out.item() == dt_ref

    # a displaced configuration, against the same formula evaluated on the host
    rng = np.random.default_rng(1)
    u = rng.uniform(-0.05, 0.05, size=p.coords.shape) / 20
    U = torch.from_numpy(u).to(dev)
    expect = float((characteristic_lengths(p.coords + u, p.conn) / np.sqrt(p.bulk_modulus / p.density)).min())
    rc = lib.nsm_critical_time_step_noalloc(p.num_nodes, p.num_elem, X.data_ptr(), U.data_ptr(), conn.data_ptr(),
                                            p.density, p.bulk_modulus, out.data_ptr(), stream)
    assert rc == 0
    torch.cuda.synchronize(dev)
    assert out.item() == expect

    # meshes beyond the fixed scratch are refused before anything runs, with a message
    rc = lib.nsm_critical_time_step_noalloc(p.num_nodes, 1048576 + 1, X.data_ptr(), None, conn.data_ptr(),
                                            p.density, p.bulk_modulus, out.data_ptr(), stream)
    assert rc == 1
    assert b"NSM_NOALLOC_MAX_ELEMENTS" in lib.nsm_last_error()
    rc = lib.nsm_critical_time_step_noalloc(p.num_nodes, p.num_elem, X.data_ptr(), None, conn.data_ptr(),
                                            -1.0, p.bulk_modulus, out.data_ptr(), stream)
    assert rc == 1 and b"positive" in lib.nsm_last_error()


def _noalloc_dt(lib, torch, p, stream, calls=2):
    """The no-allocation time step of problem p, called `calls` times in a row
    on the same output; every call must give the same value."""
    dev = torch.device("cuda:0")
    X = torch.from_numpy(np.ascontiguousarray(p.coords, dtype=np.float64).reshape(-1)).to(dev)
    conn = torch.from_numpy(np.ascontiguousarray(p.conn, dtype=np.int32).reshape(-1)).to(dev)
    out = torch.empty(1, dtype=torch.float64, device=dev)
    vals = []
    for _ in range(calls):
        out.fill_(-1.0)
        rc = lib.nsm_critical_time_step_noalloc(p.num_nodes, p.num_elem, X.data_ptr() if p.num_nodes else None,
                                                None, conn.data_ptr() if p.num_elem else None, p.density,
                                                p.bulk_modulus, out.data_ptr(), stream)
        assert rc == 0, lib.nsm_last_error()
        torch.cuda.synchronize(dev)
        vals.append(out.item())
    assert all(v == vals[0] for v in vals)
    return vals[0]


@pytest.mark.parametrize("n", [1, 65])
def test_noalloc_time_step_one_element_and_many_reduction_blocks(n):
    """One element (one partial block), and a 65^3 mesh: 274,625 elements need
    more than the 1,024 reduction blocks of 256, so the block-minimum kernel's
    grid-stride loop folds several values per thread.  Both bitwise the existing
    entry point."""
    torch = pytest.importorskip("torch")
    from nimblesm_gb300 import build as B
    from nimblesm_gb300 import engine as E
    from nimblesm_gb300.mesh import cube_problem

    B.build()
    lib = E.library()
    p = cube_problem(n, jitter=0.2 if n > 1 else 0.0, seed=11)
    model = E.Model(p)
    dt_ref = model.GetCriticalTimeStep()
    model.close()
    stream = torch.cuda.current_stream(torch.device("cuda:0")).cuda_stream
    assert _noalloc_dt(lib, torch, p, stream) == dt_ref


def test_noalloc_time_step_of_an_empty_mesh_is_the_largest_double():
    """No elements: the minimum over nothing, as nsm_critical_time_step gives an
    empty model."""
    torch = pytest.importorskip("torch")
    from nimblesm_gb300 import build as B
    from nimblesm_gb300 import engine as E

    B.build()
    lib = E.library()
    dev = torch.device("cuda:0")
    out = torch.empty(1, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for _ in range(2):
        out.fill_(-1.0)
        rc = lib.nsm_critical_time_step_noalloc(0, 0, None, None, None, 7800.0, 1.6e11, out.data_ptr(), stream)
        assert rc == 0, lib.nsm_last_error()
        torch.cuda.synchronize(dev)
        assert out.item() == np.finfo(np.float64).max


def test_noalloc_time_step_reports_a_connectivity_outside_the_mesh():
    """A connectivity entry naming a node outside [0, N) is not read: the
    element's time step is -1, and so is the result, on two calls in a row."""
    torch = pytest.importorskip("torch")
    from nimblesm_gb300 import build as B
    from nimblesm_gb300 import engine as E
    from nimblesm_gb300.mesh import cube_problem

    B.build()
    lib = E.library()
    p = cube_problem(4, jitter=0.2, seed=5)
    conn = np.ascontiguousarray(p.conn, dtype=np.int32).copy()
    conn[17, 3] = p.num_nodes  # one past the last node
    dev = torch.device("cuda:0")
    X = torch.from_numpy(np.ascontiguousarray(p.coords, dtype=np.float64).reshape(-1)).to(dev)
    C = torch.from_numpy(conn.reshape(-1)).to(dev)
    out = torch.empty(1, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for _ in range(2):
        out.fill_(0.0)
        rc = lib.nsm_critical_time_step_noalloc(p.num_nodes, p.num_elem, X.data_ptr(), None, C.data_ptr(),
                                                p.density, p.bulk_modulus, out.data_ptr(), stream)
        assert rc == 0, lib.nsm_last_error()
        torch.cuda.synchronize(dev)
        assert out.item() == -1.0

