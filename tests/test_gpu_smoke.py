import pytest

pytestmark = pytest.mark.gpu


def test_smoke_entry(gpu):
    import __graft_entry__

    __graft_entry__.smoke()
