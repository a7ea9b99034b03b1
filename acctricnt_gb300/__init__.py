"""GB300-native all-edge common-neighbour counting and SCAN queries.

The compute path is libaccx.so (hand-written sm_103a CUDA behind a C ABI,
include/accx.h); `acctricnt_gb300.accx` binds it with ctypes.
"""
import os

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libaccx.so")
CLI_PATH = os.path.join(BUILD_DIR, "scan-xp-gb300")
