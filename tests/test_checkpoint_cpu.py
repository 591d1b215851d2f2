"""MPS/MPO checkpoints in the reference's binary layout, on the host (no GPU).

The fixtures under tests/golden (*.mps, *.mpo) were written by the reference
itself (writeToFile, itensor/util/readwrite.h:363-370) from DMRG runs that
checkpoint.json records. Checked here: the library's reader and writer
reproduce those files byte for byte; the states they hold are the recorded
ones (energies through the oracle, link layouts); malformed files are
refused with ITG_ERR_ARG; and, where the reference is built (oracle/_ref),
the reference reads what the library writes and writes back the same bytes.
"""
import os
import subprocess

import pytest

from helpers import T, json_sectors, mps_energy
import mps_file

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def _files(golden):
    out = []
    for c in golden("checkpoint")["cases"]:
        out += [c["mpo"], c["start"], c["final"]]
    return out


@pytest.fixture(scope="module")
def built():
    import itensor_gb300.build as b
    return b.build()


def test_read_then_write_gives_the_reference_bytes(built, golden, tmp_path):
    import itensor_gb300 as itg
    for name in _files(golden):
        path = os.path.join(GOLDEN, name)
        f = itg.MpsFile(path)
        out = tmp_path / name
        f.write(out)
        assert out.read_bytes() == open(path, "rb").read(), name


def test_file_info_matches_the_recorded_runs(built, golden):
    import itensor_gb300 as itg
    for c in golden("checkpoint")["cases"]:
        names = ["Nf", "Sz"] if c["model"]["type"] == "hubbard" else ["Sz"]
        for key, lims in (("start", c["start_lims"]), ("final", c["final_lims"])):
            info = itg.MpsFile(os.path.join(GOLDEN, c[key])).info()
            assert info["nsites"] == c["N"]
            assert [info["leftlim"], info["rightlim"]] == lims
            assert info["qn_names"] == names
        assert itg.MpsFile(os.path.join(GOLDEN, c["mpo"])).info()["nsites"] == c["N"]


def test_reference_files_hold_the_recorded_states(golden):
    """Independent reader + oracle: the start state's energy is the first run's,
    the final state's the continued run's (both after truncation, so to 1e-8),
    and the link layouts are the recorded ones."""
    for c in golden("checkpoint")["cases"]:
        W, _, _ = mps_file.read(os.path.join(GOLDEN, c["mpo"]))
        Wt = [T(x) for x in W]
        for key, energy, links in (("start", c["start_energy"], c["start_links"]),
                                   ("final", c["energy"], c["links"])):
            psi, _, _ = mps_file.read(os.path.join(GOLDEN, c[key]))
            assert abs(mps_energy([T(x) for x in psi], Wt) - energy) < 1e-8, (c["name"], key)
            for j, ref in enumerate(links):
                common = [I for I in psi[j]["inds"] if I["id"] in {J["id"] for J in psi[j + 1]["inds"]}]
                assert len(common) == 1
                assert json_sectors(common[0]) == json_sectors(ref)


def test_malformed_files_are_refused(built, golden, tmp_path):
    import itensor_gb300 as itg
    src = open(os.path.join(GOLDEN, golden("checkpoint")["cases"][0]["start"]), "rb").read()
    cases = {"truncated.mps": src[: len(src) // 2], "trailing.mps": src + b"\0\0\0\0", "empty.mps": b"",
             "bad_count.mps": src[:4] + b"\xff" * 8 + src[12:]}
    for name, data in cases.items():
        p = tmp_path / name
        p.write_bytes(data)
        with pytest.raises(itg.ITGError) as e:
            itg.MpsFile(p)
        assert e.value.code == 1, name
    with pytest.raises(itg.ITGError) as e:
        itg.MpsFile(tmp_path / "missing.mps")
    assert e.value.code == 1


def test_the_reference_reads_what_the_library_writes(built, golden, tmp_path):
    """readFromFile + writeToFile of the reference on the library's output give
    the same bytes (where the reference is built in this container)."""
    ref = os.path.join(ROOT, "oracle", "_ref", "ref_golden")
    if not os.path.exists(ref):
        pytest.skip("the reference is not built here (oracle/_ref)")
    import itensor_gb300 as itg
    for name in _files(golden):
        ours = tmp_path / ("ours_" + name)
        itg.MpsFile(os.path.join(GOLDEN, name)).write(ours)
        back = tmp_path / ("ref_" + name)
        subprocess.run([ref, "--rewrite", str(ours), str(back)], check=True, capture_output=True,
                       env=dict(os.environ, OMP_NUM_THREADS="1"))
        assert back.read_bytes() == ours.read_bytes(), name
