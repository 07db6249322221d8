"""Where the in-tree shared libraries live."""
import os

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)            # dials-metal_gb300/
CSRC = os.path.join(ROOT, "csrc")
HOST = os.path.join(ROOT, "host")
REPO = os.path.dirname(ROOT)
INCLUDE = os.path.join(REPO, "include")


def core_lib() -> str:
    return os.path.join(PKG_DIR, "libsfgb.so")


def synth_lib() -> str:
    return os.path.join(PKG_DIR, "libsfsynth.so")
