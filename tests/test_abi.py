"""The C-ABI library loads and exports every symbol the public headers
declare (no GPU needed: nothing here launches work)."""
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:int|long long|int64_t|double|void)\s+\**(lgd_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def library():
    import __graft_entry__
    __graft_entry__.build()
    from libgeodecomp_gb300 import lgd
    return lgd.lib()


def test_headers_declare_entry_points():
    assert len(declared_symbols()) >= 20


@pytest.mark.parametrize("name", declared_symbols())
def test_symbol_exported(library, name):
    assert hasattr(library, name), name


def test_version_and_device_count_without_gpu(library):
    from libgeodecomp_gb300 import lgd
    assert library.lgd_gpu_version() >= 10000
    assert lgd.device_count() >= 0


def test_create_reports_error_code_not_crash(library):
    """Without a usable device (or with a bad descriptor) create returns a
    status code and a message instead of throwing across the ABI."""
    from libgeodecomp_gb300 import lgd
    with pytest.raises(lgd.LGDError) as e:
        lgd.Grid(lgd.CELL_JACOBI7_F64, (0, 4, 4))
    assert e.value.code in (lgd.ERR_INVALID, lgd.ERR_CUDA)
    with pytest.raises(lgd.LGDError):
        lgd.Grid(999, (4, 4, 4))


def test_snapshot_info_reads_the_reference_header(tmp_path):
    """lgd_snapshot_info (host only) reads the header of the reference's
    MPIIO layout (io/mpiio.h:70-79 readMetadata): DIM int32, step, maximum."""
    import struct
    from libgeodecomp_gb300 import lgd
    p = tmp_path / "h00007.mpiio"
    p.write_bytes(struct.pack("<3i2I", 12, 9, 7, 7, 21) + struct.pack("<d", 0.25) + bytes(8 * 12 * 9 * 7))
    assert lgd.snapshot_info(str(p), 3) == ((12, 9, 7), 7, 21)
    p2 = tmp_path / "h2.mpiio"
    p2.write_bytes(struct.pack("<2i2I", 64, 40, 3, 5) + bytes(1 + 64 * 40))
    assert lgd.snapshot_info(str(p2), 2) == ((64, 40), 3, 5)
    p3 = tmp_path / "short.mpiio"
    p3.write_bytes(struct.pack("<3i", 1, 2, 3))
    with pytest.raises(lgd.LGDError):
        lgd.snapshot_info(str(p3), 3)
