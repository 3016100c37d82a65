"""The reference's own example decks (Examples/1D/Euler1D, 2D/Euler2D, 3D/NavierStokes3D,
one level of sub-decks) through the deck reader, where the reference's source tree is
present (HYPAR_REF, else the path the build uses).  Each deck is copied with a stand-in
initial solution of the right shape where its aux program would write one; every deck
must read, except those that need what is outside the WENO path (an immersed body, a
libROM prediction, MUSCL3: GB_ERR_UNSUPPORTED) or a file that only its aux program
writes (GB_ERR_INPUT).  CPU only: the reader, no device."""
import glob
import os
import shutil

import numpy as np
import pytest

from hypar_gb300 import _lib
from hypar_gb300.solver import Inputs


def _ref_examples():
    import __graft_entry__ as g
    root = os.environ.get("HYPAR_REF") or g.REFERENCE
    return os.path.join(root, "Examples")


EX = _ref_examples()
pytestmark = pytest.mark.skipif(not os.path.isdir(EX), reason="the reference's source tree is not present")

# (deck name part, expected error code): refusals with their reason
REFUSED = [("immersed", 4),                      # solver.inp immersed_body: not on this path
           ("2D_Shock_Cylinder_Interaction", 4),  # immersed body
           ("2D_Cylinder/", 4), ("Sphere/", 4),
           ("libROM_DMD_Predict", 4),            # hyp_space_scheme 1: a ROM surrogate
           ("2D_RiemannCase4/", 4),              # MUSCL3
           ("RisingThermalBubble_Config1_CUDA", 3),  # parallel input files its aux program writes
           ("SteadyWarmGround", 3), ("SupersonicHotChannelFlow", 3)]  # wall temperature files from aux


def _decks():
    if not os.path.isdir(EX):
        return []
    found = set()
    for sub in ("1D/Euler1D", "2D/Euler2D", "3D/NavierStokes3D"):
        for d in glob.glob(os.path.join(EX, sub, "*")) + glob.glob(os.path.join(EX, sub, "*", "*")):
            if os.path.isfile(os.path.join(d, "solver.inp")):
                found.add(os.path.relpath(d, EX))
    return sorted(found)


def _stand_in_initial(d):
    """An initial.inp of the deck's size (x then the conserved variables, uniform
    state) where the deck has none, in its ip_file_type."""
    if os.path.exists(os.path.join(d, "initial.inp")):
        return
    toks = open(os.path.join(d, "solver.inp")).read().split()
    nd = int(toks[toks.index("ndims") + 1])
    nv = int(toks[toks.index("nvars") + 1])
    i = toks.index("size")
    size = [int(t) for t in toks[i + 1:i + 1 + nd]]
    ipt = toks[toks.index("ip_file_type") + 1] if "ip_file_type" in toks else "ascii"
    xs = np.concatenate([np.linspace(0.0, 1.0, n) for n in size])
    u = np.zeros((int(np.prod(size)), nv))
    u[:, 0] = 1.0
    u[:, -1] = 2.5
    if ipt in ("bin", "binary"):
        open(os.path.join(d, "initial.inp"), "wb").write(xs.tobytes() + u.tobytes())
    else:
        with open(os.path.join(d, "initial.inp"), "w") as f:
            f.write(" ".join(repr(float(v)) for v in xs) + "\n")
            for v in range(nv):
                f.write(" ".join(repr(float(a)) for a in u[:, v]) + "\n")


@pytest.mark.parametrize("name", _decks())
def test_reference_example_deck_reads(built_lib, tmp_path, name):
    d = str(tmp_path / "deck")
    shutil.copytree(os.path.join(EX, name), d)
    _stand_in_initial(d)
    want = [code for part, code in REFUSED if part in name + "/"]
    if want:
        with pytest.raises(_lib.GbError) as e:
            Inputs(d)
        assert e.value.code == want[0], str(e.value)
    else:
        inp = Inputs(d)
        assert inp.config.nvars in (3, 4, 5)


def test_reference_gravity_decks_are_covered():
    """The decks that need gravity with CRWENO5 and the 1-D slip wall are among those
    that read (not refused)."""
    names = _decks()
    for n in ("1D/Euler1D/SodShockTubeWithGravity", "1D/Euler1D/SmallPerturbationWithGravity_02"):
        assert n in names
        assert not any(part in n + "/" for part, _ in REFUSED)
