"""Errors of the command-line front end (gpucsl/cli/cli_util.py:5-19): an error is logged
and raised as GpucslError, which `python -m gpucsl_gb300` turns into exit status 1."""
from __future__ import annotations

import logging


class GpucslError(Exception):
    pass


def error(message: str):
    logging.error(message)
    raise GpucslError(message)


def warning(message: str):
    logging.warning(message)
