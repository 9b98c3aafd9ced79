"""``python -m fgrain_gb300 ...``: the fgrain command line (src/main.rs)."""
import sys

from .cli import main

sys.exit(main())
