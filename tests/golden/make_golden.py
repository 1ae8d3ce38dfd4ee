"""Copies the reference's own golden vector for the lid-driven-cavity regression
(tests/lid_driven_cavity/data_ldc_re1000.txt of the SNaC source tree: 64 rows of
z-coordinate and v-velocity after 1500 steps) into tests/golden/, so that the
tests can run where the reference tree is absent.

Usage: python tests/golden/make_golden.py /path/to/SNaC
"""
import os
import shutil
import sys

if len(sys.argv) != 2:
    sys.exit("usage: python tests/golden/make_golden.py /path/to/SNaC")
src_root = sys.argv[1]
here = os.path.dirname(os.path.abspath(__file__))
shutil.copyfile(os.path.join(src_root, "tests", "lid_driven_cavity", "data_ldc_re1000.txt"),
                os.path.join(here, "ldc_re1000_profile.txt"))
print("wrote", os.path.join(here, "ldc_re1000_profile.txt"))
