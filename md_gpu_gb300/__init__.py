"""md_gpu_gb300: md_gpu's per-step force-and-integrate path as hand-written
sm_103a CUDA kernels behind a C ABI (include/md_gpu.h).

    from md_gpu_gb300 import MDSystem
    sim = MDSystem.from_files("run/nacl")     # <base>.inp/.fld/.cfg
    sim.step(1000)
    print(sim.thermo())
"""
from .system import (MDError, MDSystem, MD_LEAPFROG, MD_NH, MD_VV, TERM_ALL, TERM_ANGLE,  # noqa: F401
                     TERM_BOND, TERM_PAIR, TERM_RECIP, fp32_peak_tflops, library)
