"""Argument checks of the public API (gpucsl/pc/pc_validations.py, gpucsl/cli/cli_util.py)."""
from __future__ import annotations

import logging


class GpucslError(Exception):
    """User-facing error (gpucsl/cli/cli_util.py:5-11)."""


def error(message: str):
    raise GpucslError(message)


def warning(message: str):
    logging.warning(message)


def validate_alpha(alpha):
    """pc_validations.py:25-27."""
    if alpha < 0 or alpha > 1:
        error("Alpha level has to be between 0 and 1")


def validate_given_devices(devices, sync_device):
    """This build is single-GPU: only one device may be named (the reference's
    multi-GPU device manager is not part of it)."""
    if devices is None or len(devices) != 1:
        error(f"gpucsl_gb300 runs one skeleton per GPU; give exactly one device, not {devices}")
    if sync_device is not None and sync_device not in devices:
        error(f"The sync device has to be one of the specified gpus. You gave gpus: {devices} "
              f"and sync device: {sync_device}")


def determine_max_level(max_level, data):
    """None -> p - 2; larger values are clamped to p - 2 (pc_validations.py:45-61)."""
    variable_count = data.shape[1]
    max_possible_level = variable_count - 2
    if max_level is None:
        max_level = max_possible_level
        if max_level < 0:
            error(f"Max level should be >= 0. Your input: {max_level}")
    if max_level > max_possible_level:
        warning(f"You set the max level to {max_level}, but the biggest possible level is "
                f"{max_possible_level}. The pc algorithm will at a maximum only run until level "
                f"{max_possible_level}.")
        max_level = max_possible_level
    return max_level
