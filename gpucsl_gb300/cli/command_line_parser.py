"""The reference's command line (gpucsl/cli/command_line_parser.py:4-70): same short and
long options, defaults and required arguments."""
from __future__ import annotations

import argparse


def build_command_line_parser() -> argparse.ArgumentParser:
    ap = argparse.ArgumentParser(description="Causal structure learning (PC-stable) on a GB300.")
    ap.add_argument("-a", "--alpha", type=float, default=0.05, help="significance level of the CI tests")
    ap.add_argument("-b", "--debug", action="store_true",
                    help="accepted for compatibility (the kernels are compiled ahead of time)")
    ap.add_argument("-c", "--correlation-matrix", help="path of a cached correlation matrix (CSV)")
    ap.add_argument("-d", "--dataset", default="", required=True, help="samples (CSV, one row per sample)")
    ap.add_argument("--discrete", action="count", default=0, help="discrete (chi-squared) CI tests")
    ap.add_argument("--gaussian", action="count", default=0, help="Gaussian (Fisher z) CI tests")
    ap.add_argument("-g", "--gpus", type=int, nargs="+",
                    help="GPU indices; one GPU is used (the first given, else the current device)")
    ap.add_argument("-l", "--max-level", type=int, help="largest separating-set size")
    ap.add_argument("-o", "--output-directory", required=True, help="directory of the output files")
    ap.add_argument("-s", "--sync-device", type=int, help="accepted for compatibility (single GPU)")
    ap.add_argument("-v", "--verbose", action="count", default=0, help="-v: info, -vv: debug logging")
    return ap
