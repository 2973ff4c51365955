"""SortingCallback host logic (CPU): argument checks of the reference's constructor
(src/callbacks/sorting.jl:36-55) and the oracle's permutation = Julia's stable sortperm over the
lexicographic cell coordinates."""
import numpy as np
import pytest

from helpers import dam_break_case


def test_sorting_callback_arguments(pkg):
    with pytest.raises(ValueError, match="ArgumentError"):
        pkg.SortingCallback(interval=3, dt=0.1)
    with pytest.raises(ValueError, match="ArgumentError"):
        pkg.SortingCallback()
    cb = pkg.SortingCallback(interval=3)
    assert cb.interval == 3 and cb.dt is None and cb.initial_sort and not cb.sort_masses
    cb = pkg.SortingCallback(dt=0.01, initial_sort=False)
    assert cb.interval is None and cb.dt == 0.01 and not cb.initial_sort


@pytest.mark.parametrize("nd", [2, 3])
def test_oracle_sort_perm_is_lexicographic_stable(pkg, orc, nd):
    if nd == 2:
        semi, tank = dam_break_case(pkg, 2, 0.05, (1.0, 0.5), (2.0, 1.0), jitter=0.3, seed=8)
    else:
        semi, tank = dam_break_case(pkg, 3, 0.08, (0.6, 0.3, 0.6), (1.2, 0.6, 0.8), jitter=0.3,
                                    seed=8)
    x = tank.fluid.coordinates.copy()
    rng = np.random.default_rng(1)
    x = x[rng.permutation(x.shape[0])]
    perm = orc.sort_perm(semi.config, x)
    cs = 2.0 * semi.config.smoothing_length
    c = np.floor(x / cs).astype(np.int64)
    keys = [c[:, d] for d in reversed(range(nd))]  # lexsort: last key is the primary one
    assert np.array_equal(perm, np.lexsort(keys))
