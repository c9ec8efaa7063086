import os
import sys

# the reference's whole-path PotEnergy races on a shared dr[3] under OpenMP
# (mc_piqmc.cc:1210,1237); the compiled reference is run single-threaded
os.environ.setdefault("OMP_NUM_THREADS", "1")

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
for p in (HERE, os.path.join(REPO, "oracle"), os.path.join(REPO, "moribs-pimc_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
