"""The recipes under oracle/ref compile the reference's own sources where
they lie; on a machine without the reference checkout (the GPU machine) they
must exit 3, which build() takes as "keep the prebuilt files", and nothing
else. Each recipe takes the root from its argument, else CCP_REFERENCE_ROOT."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
RECIPES = ("build_ref.sh", "build_sostat.sh", "build_chrana.sh", "build_ccp_programs.sh")


@pytest.mark.parametrize("recipe", RECIPES)
def test_recipe_without_checkout_exits_3(recipe, tmp_path):
    path = os.path.join(ROOT, "oracle", "ref", recipe)
    missing = str(tmp_path / "no-such-checkout")
    r = subprocess.run([path, missing], capture_output=True, text=True)
    assert r.returncode == 3, (r.returncode, r.stderr)
    assert "no reference checkout" in r.stderr
    env = dict(os.environ, CCP_REFERENCE_ROOT=missing)
    r = subprocess.run([path], capture_output=True, text=True, env=env)
    assert r.returncode == 3, (r.returncode, r.stderr)


def test_build_entry_treats_exit_3_as_absent():
    import __graft_entry__ as g

    assert g.RECIPE_NO_REFERENCE == 3
