"""`python -m gpucsl_gb300 -d data.csv --gaussian -l 3 -o out/` (gpucsl/cli/cli.py:20-96):
read the samples (and a cached correlation matrix), run GaussianPC / DiscretePC on the
GPU, write the CPDAG, separating sets, pmax and the command line."""
from __future__ import annotations

import logging

from .cli_io import read_correlation_matrix, read_csv, write_results_and_config
from .cli_util import error
from .command_line_parser import build_command_line_parser
from ..pc.pc import DiscretePC, GaussianPC


def _log_level(verbose: int):
    if verbose == 1:
        logging.basicConfig(level=logging.INFO)
    elif verbose > 1:
        logging.basicConfig(level=logging.DEBUG)


def gpucsl_cli(command_line_arguments):
    args = build_command_line_parser().parse_args(command_line_arguments)
    _log_level(args.verbose)
    if args.gaussian + args.discrete != 1:
        error("Please set exactly one of the options --gaussian/--discrete")
    if args.discrete and args.correlation_matrix is not None:
        error("Discrete independence test does not use a correlation matrix. Please check the arguments.")
    gpus = args.gpus
    if args.discrete and gpus is not None and len(gpus) > 1:
        error("Multi GPU independence tests are only supported for the gaussian independence test")
    if gpus is not None and len(gpus) > 1:
        error("This build solves a skeleton on one GPU: give at most one index with -g")
    if gpus:
        import torch

        torch.cuda.set_device(gpus[0])
    data = read_csv(args.dataset)
    should_log = args.verbose > 0
    if args.discrete:
        pc = DiscretePC(data, args.max_level, args.alpha, is_debug=args.debug, should_log=should_log)
        pc.set_distribution_specific_options()
    else:
        pc = GaussianPC(data, args.max_level, args.alpha, is_debug=args.debug, should_log=should_log)
        device = [gpus[0]] if gpus else [0]
        pc.set_distribution_specific_options(device, None, read_correlation_matrix(args.correlation_matrix))
    result = pc.execute().result  # timings are for benchmarks only
    write_results_and_config(args.output_directory, args.dataset, command_line_arguments, result)
    return result
