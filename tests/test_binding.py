"""The reference-side binding (opencaeporox_gb300/binding/
IsoThermalMethodGPU.hpp), compiled against the reference's own headers and
linked to the library by oracle/ref/Makefile, driven on the black-oil deck of
the 10 x 10 x 3 configuration and on a six-component PR-EoS deck set up by the
reference's IsothermalSolver.  The binding describes the reference's model and
grid to the library; on a host without a CUDA device the library checks the
descriptions and answers OCPX_NO_DEVICE, which the binding reports as such.
Needs the reference's sources (skipped where they are absent)."""
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))


def _binding():
    from oracle import build as ob
    if not os.path.isdir(os.path.join(ob.REF, "src")):
        pytest.skip("the reference's sources are not on this machine")
    from opencaeporox_gb300 import build
    build.build()
    return ob.build_binding()


@pytest.mark.parametrize("case", ["blackoil", "comp6"])
def test_binding_describes_the_reference_model(tmp_path, case):
    import decks
    exe = _binding()
    if case == "blackoil":
        text, nb, nconn, nc, mixture = decks.blackoil_deck(seed=1), 300, 740, 3, 0
    else:
        ni, text = decks.comp_deck(4, 3, 2, 6, seed=2)
        nb, nconn, nc, mixture = 24, 4 * 3 * 2 * 3 - 4 * 2 - 3 * 2 - 4 * 3, 7, 1
    deck = tmp_path / "case.data"
    deck.write_text(text)
    if case != "blackoil":
        ni.astype("<f8").tofile(str(deck) + ".ptn_ni")   # PTN moles, as the fixture generator passes them
    r = subprocess.run([exe, str(deck)], capture_output=True, text=True, timeout=300, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert f"description nb {nb} nbI {nb} nconn {nconn} nc {nc} mixture {mixture}" in r.stdout, r.stdout
    # this machine has no CUDA device: the descriptions passed the library's checks
    assert "status OCPX_NO_DEVICE" in r.stdout or "status OCPX_OK" in r.stdout, r.stdout


@pytest.mark.parametrize("case", ["blackoil", "comp6"])
def test_binding_recompute_option(tmp_path, case):
    """IsoT_FIM_GPU::SetRecomputeFlashDer: a compositional deck passes the
    library's checks with the option (OCPX_NO_DEVICE here), a black-oil deck
    is refused (it has no flash to recompute from)."""
    import decks
    exe = _binding()
    deck = tmp_path / "case.data"
    if case == "blackoil":
        deck.write_text(decks.blackoil_deck(seed=1))
    else:
        ni, text = decks.comp_deck(4, 3, 2, 6, seed=2)
        deck.write_text(text)
        ni.astype("<f8").tofile(str(deck) + ".ptn_ni")
    r = subprocess.run([exe, str(deck), "--recompute"], capture_output=True, text=True, timeout=300, cwd=tmp_path)
    if case == "blackoil":
        assert r.returncode == 2 and "OCPX_INVALID_ARG" in r.stdout and "compositional" in r.stdout, r.stdout
    else:
        assert r.returncode == 0, r.stdout + r.stderr
        assert "status OCPX_NO_DEVICE" in r.stdout or "status OCPX_OK" in r.stdout, r.stdout
