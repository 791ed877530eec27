"""The entry point's smoke check (one small persistent ATsit5 solve against the
oracle) runs as part of the GPU suite, so that it stays green."""
import pytest

pytestmark = pytest.mark.gpu


def test_entry_smoke():
    import __graft_entry__ as g
    g.smoke()
