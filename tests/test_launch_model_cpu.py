"""Host-side launch decisions of the subsampling kernels, compiled with the
host compiler from octree-cuda_gb300/csrc/kernels.h (no GPU): the cluster size
of distance-weighted levels from the device's cluster slots."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")

# clusters of 2, 4, 8, 16 subsample blocks one GB300 held at once (76, 36, 15, 7),
# and a chip that holds only 3 clusters of 16
GB300 = [0, 76, 36, 15, 7]
FEW16 = [0, 76, 36, 15, 3]
CASES = [
    # slots, nodes, SMs, balance, cap -> cluster size
    (GB300, 300, 152, 16, 16, 16),   # many nodes, the largest a tenth of the level
    (GB300, 300, 152, 8, 16, 8),
    (GB300, 300, 152, 4, 16, 4),
    (FEW16, 300, 152, 16, 16, 8),    # fewer clusters of 16: smaller clusters
    (GB300, 1, 152, 64, 16, 16),     # the root
    (GB300, 300, 152, 16, 4, 4),     # the cap
    (GB300, 1, 1, 64, 16, 1),        # the allocation-free entry point: one block
]


@pytest.mark.skipif(not shutil.which("g++") or not os.path.exists(CUDA_INC), reason="no host compiler or CUDA headers")
def test_weighted_cluster_choice(tmp_path):
    body = []
    for k, (slots, n, sms, bal, cap, _) in enumerate(CASES):
        body.append("{ const int s[5] = {%s}; std::printf(\"%%u\\n\", oc::weighted_cluster_choice(s, %du, %d, %du, %du)); }"
                    % (", ".join(map(str, slots)), n, sms, bal, cap))
    src = tmp_path / "choice.cpp"
    src.write_text('#include <cstdio>\n#include "kernels.h"\nint main() {\n' + "\n".join(body) + "\nreturn 0;\n}\n")
    exe = tmp_path / "choice"
    subprocess.run(["g++", "-std=c++17", "-I", CUDA_INC, "-I", os.path.join(ROOT, "octree-cuda_gb300", "csrc"),
                    str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert got == [c[-1] for c in CASES]
