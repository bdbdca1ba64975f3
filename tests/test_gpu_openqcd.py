"""openQCD gauge files (Grid/parallelIO/OpenQcdIO.h) through the library's device reader
against the oracle's numpy writer: the field comes back bit-exact, the header plaquette is
converted to Grid's normalisation and checked; a wrong plaquette is refused."""
import numpy as np
import pytest

import grid_gb300 as g
from oracle import nersc, openqcd

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims", [(4, 4, 4, 8), (6, 4, 8, 4)])
def test_read_oracle_file(gpu_available, tmp_path, dims):
    U = g.random_gauge(dims, 0.5, 121)
    path = tmp_path / "cfg.oq"
    plaq = openqcd.write(path, U, dims)
    V, d, p_file, p_comp = g.openqcd_read(path)
    assert d == tuple(dims)
    assert np.array_equal(V, U)
    assert abs(p_file - plaq) < 1e-15 and abs(p_comp - plaq) < 2e-15
    assert abs(p_comp - nersc.plaquette_and_trace(U, dims)[0]) < 2e-15


def test_wrong_plaquette_is_refused(gpu_available, tmp_path):
    dims = (4, 4, 4, 4)
    U = g.random_gauge(dims, 0.5, 122)
    path = tmp_path / "bad.oq"
    openqcd.write(path, U, dims, plaquette=0.5)
    with pytest.raises(g.GridError):
        g.openqcd_read(path)
    V, _, _, _ = g.openqcd_read(path, check=False)
    assert np.array_equal(V, U)
