"""Wavefunction files and InitialConditionType.File (Problem.py:397-474, serialization/Pickle.py):
pickled data arrays (protocol 2) and two-column ASCII, written and read back exactly, as the
initial condition of a second problem on the same grid; a shape mismatch is refused."""
import numpy as np
import pytest

from helpers import config_text


def _problem(text):
    import pyprop_gb300 as pp
    prob = pp.Problem(pp.LoadString(text), device="cpu")
    prob.SetupWavefunction()
    return prob


def _file_ic(text, fmt, path):
    i = text.index("[InitialCondition]")
    j = text.index("[", i + 1)
    return (text[:i] + "[InitialCondition]\ntype = InitialConditionType.File\nformat = WavefunctionFileFormat.%s\n"
            "filename = \"%s\"\n\n" % (fmt, path) + text[j:])


@pytest.mark.parametrize("fmt,suffix", [("Binary", "pickle"), ("Ascii", "txt")])
def test_save_and_start_from_file(tmp_path, fmt, suffix):
    text = config_text(maxl=3, xsize=30, m=8)
    src = _problem(text)
    path = str(tmp_path / ("psi." + suffix))
    if fmt == "Binary":
        src.SaveWavefunctionPickle(path)
    else:
        src.SaveWavefunctionAscii(path)
    dst = _problem(_file_ic(text, fmt, path))
    assert np.array_equal(dst.psi.GetDataNumpy(), src.psi.GetDataNumpy())


def test_loaded_shape_must_match(tmp_path):
    small = _problem(config_text(maxl=3, xsize=30, m=8))
    path = str(tmp_path / "psi.pickle")
    small.SaveWavefunctionPickle(path)
    other = _problem(config_text(maxl=4, xsize=30, m=8))
    with pytest.raises(ValueError, match="Invalid shape"):
        other.LoadWavefunctionPickle(path)


def test_hdf_format_is_reported_unavailable(tmp_path):
    text = config_text(maxl=3, xsize=30, m=8)
    with pytest.raises(NotImplementedError, match="HDF5"):
        _problem(_file_ic(text, "HDF", str(tmp_path / "psi.h5")).replace(
            "format = WavefunctionFileFormat.HDF\n", "format = WavefunctionFileFormat.HDF\ndataset = \"/wavefunction\"\n"))
