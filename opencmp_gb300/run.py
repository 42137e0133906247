"""``run(config_file_path, config_parser=None)``: OpenCMP's entry point (``opencmp/run.py:30-71``)
on the GPU path. Loads the configuration, looks up the model and solver classes, solves, and then
runs OpenCMP's post-processing (``opencmp/post_processing/__init__.py:28-43``): the error metrics and
the h / p convergence tests."""
from __future__ import annotations

from typing import Optional

from .config import ConfigParser
from .models import get_model_class
from .post_processing import run_post_processing
from .solvers import get_solver_class


def run(config_file_path: str, config_parser: Optional[ConfigParser] = None):
    if config_parser is None:
        config_parser = ConfigParser(config_file_path)
    elif not isinstance(config_parser, ConfigParser):
        config_parser = ConfigParser.from_parser(config_parser)   # e.g. OpenCMP's own parser
    model_name = config_parser.get_item(['OTHER', 'model'], str)
    dim_used = config_parser.get_item(['DIM', 'diffuse_interface_method'], bool, quiet=True)
    model_class = get_model_class(model_name, dim_used)
    solver_class = get_solver_class(config_parser)
    solver = solver_class(model_class, config_parser)
    sol = solver.solve()
    run_post_processing(config_parser, solver, sol)
    return solver, sol
