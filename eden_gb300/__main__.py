"""python -m eden_gb300 nml <LEMS file> [rng_seed N] [verbose] [plain]"""
import sys

from .cli import main

sys.exit(main())
