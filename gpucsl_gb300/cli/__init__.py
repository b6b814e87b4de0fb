"""Command-line front end with the reference's options and output files
(gpucsl/cli/: cli.py, cli_io.py, command_line_parser.py, cli_util.py)."""
