"""`python -m gpucsl_gb300 ...`: the command line of gpucsl/__main__.py (no stack trace for
usage errors, exit status 1)."""
import sys

from .cli.cli import gpucsl_cli
from .cli.cli_util import GpucslError

if __name__ == "__main__":
    try:
        gpucsl_cli(sys.argv[1:])
    except GpucslError:
        sys.exit(1)
