"""`python -m em_lab_gb300 --script scene.lua --frames N`: the headless scene runner."""
import sys

from .headless import main

sys.exit(main())
