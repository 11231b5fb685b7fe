"""The build's smoke entry point (__graft_entry__.smoke) as a GPU test: one
small RPD through the C ABI checked against the oracle, then the default
engine (certified cells, exact lists) on short lists."""
import pytest

import __graft_entry__ as entry

pytestmark = pytest.mark.gpu


def test_smoke_entry_point():
    entry.smoke()
