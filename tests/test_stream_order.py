"""Setup uploads are in device memory before any operator kernel runs.

The operators run on non-blocking streams, which do not wait for the legacy
stream. A plain cudaMemcpy from pageable host memory returns once the data is
staged, with its DMA possibly still running on the legacy stream, and a
cudaMemset is asynchronous on it: a kernel launched next on an operator's
stream could read the buffer before it is written. With many operators'
streams busy at once (the ensemble), such a kernel read uninitialised system
descriptors and offsets. Every host-to-device copy and memset of the operator
code therefore goes through CopyIn / ZeroIn (common.cuh), which wait for the
legacy stream, or is stream-ordered (cudaMemcpyAsync / cudaMemsetAsync on the
operator's stream). The band solvers' host-pointer entry points (band.cu) run
their kernels on the legacy stream itself and may copy on it."""

import pathlib
import re

CSRC = pathlib.Path(__file__).resolve().parent.parent / "sl3dpp_gb300" / "csrc"
LEGACY_STREAM_FILES = {"band.cu"}  # copies and kernels all on the legacy stream


def _calls(text, name):
    return [m.start() for m in re.finditer(r"\b" + name + r"\s*\(", text)]


def test_no_unordered_uploads_in_operator_code():
    offenders = []
    for path in sorted(CSRC.rglob("*.cu")) + sorted(CSRC.rglob("*.cuh")):
        if path.name in LEGACY_STREAM_FILES:
            continue
        text = path.read_text()
        for pos in _calls(text, "cudaMemcpy"):
            call = text[pos:text.index(";", pos)]
            if "cudaMemcpyHostToDevice" in call or "cudaMemcpyDeviceToDevice" in call:
                if path.name == "common.cuh" and "CopyIn" in text[max(0, pos - 400):pos]:
                    continue  # the helper itself
                offenders.append(f"{path.name}:{text.count(chr(10), 0, pos) + 1}")
        for pos in _calls(text, "cudaMemset"):
            if path.name == "common.cuh":
                continue  # ZeroIn itself
            offenders.append(f"{path.name}:{text.count(chr(10), 0, pos) + 1}")
    assert not offenders, "unordered host-to-device copies or memsets: " + ", ".join(offenders)


def test_upload_helper_waits_for_the_legacy_stream():
    text = (CSRC / "common.cuh").read_text()
    body = text[text.index("inline cudaError_t CopyIn"):]
    body = body[:body.index("\n}\n")]
    assert "cudaStreamSynchronize(cudaStreamLegacy)" in body
    assert "CopyIn(p, v.data()" in (CSRC / "systems.cuh").read_text()
