"""The continuous-batching server keeps its cohorts and jobs in lists and
removes finished ones with list.remove: the records must compare by
identity, not field by field (their fields hold arrays, whose == has no
single truth value).  Host logic only; no device is touched."""
import numpy as np
import pytest

pytest.importorskip("torch")

from laml_gb300 import serving as S  # noqa: E402


def _cohort(k):
    return S._Cohort(jobs=[], batch=None, stream=None, kind="em", footprint=k, event=None,
                     done=np.zeros(3, bool), host_status=None)


def test_cohorts_compare_by_identity():
    a, b, c = _cohort(1), _cohort(1), _cohort(1)
    active = [a, b, c]
    active.remove(c)          # compares a and b with c first
    assert active == [a, b] and a != b
    assert S._replace_cohort(active, b, c) is c and active == [a, c]


def test_jobs_compare_by_identity():
    j1 = S._Job(req=None, tree=None, ds=None, footprint=1, future=None, t_submit=0.0)
    j2 = S._Job(req=None, tree=None, ds=None, footprint=1, future=None, t_submit=0.0)
    assert j1 != j2 and [j1, j2].index(j2) == 1
