"""Post-processing of a run: OpenCMP's error metrics and its convergence tests
(``opencmp/post_processing/__init__.py:28-43``, ``opencmp/post_processing/error_analysis.py:28-161``).

``[ERROR ANALYSIS] convergence_test = h -> u`` re-solves the problem on ``num_refinements``
uniformly refined meshes (every triangle into four, every tetrahedron into eight,
``mesh.refine_uniform``); ``p -> u`` re-solves it with the interpolant order raised by one each
time. Each prints ``L2 norm at refinement <n>: <error>`` and then the table OpenCMP prints, with
its rate formulas: h: log(e_n / e_{n+1}) / log(N_{n+1} / (N_n 2^(D-1))) over the element counts N;
p: log(e_n / e_{n+1}) / log(n_{n+1} / n_n) over the dof counts n. The table is drawn by ``tabulate``
where it is installed (OpenCMP's choice) and in the same columns and number formats otherwise.
"""
from __future__ import annotations

import math
from typing import List, Sequence

from .config import ConfigParser
from .mesh import refine_uniform


def run_post_processing(config_parser: ConfigParser, solver, sol) -> None:
    """OpenCMP's ``run_post_processing``: the error metrics, then the convergence tests."""
    if config_parser.get_item(['ERROR ANALYSIS', 'check_error'], bool):
        solver.report()
    convergence_analysis(config_parser, solver, sol)


def _tests(config_parser: ConfigParser):
    if not config_parser.has_option('ERROR ANALYSIS', 'convergence_test'):
        return {}
    raw = config_parser.get_dict(['ERROR ANALYSIS', 'convergence_test'], all_str=True)
    out = {}
    for key, val in raw.items():
        names = [v.strip() for v in str(val).split(',') if v.strip() and v.strip() != 'False']
        out[key.strip()] = names
    return out


def convergence_analysis(config_parser: ConfigParser, solver, sol) -> None:
    for key, names in _tests(config_parser).items():
        if key == 'h':
            for var in names:
                h_convergence(config_parser, solver, sol, var)
        elif key == 'p':
            for var in names:
                p_convergence(config_parser, solver, sol, var)
        elif names:
            raise ValueError('convergence_test: unknown test {!r} (h or p)'.format(key))


def _check_average(config_parser: ConfigParser, var: str) -> None:
    average = config_parser.get_list(['ERROR ANALYSIS', 'error_average'], str, quiet=True)
    if var in average:
        raise NotImplementedError('error_average (the mean-free L2 error) is not on the GPU path')


def _resolve(solver, config: ConfigParser):
    """A new solver of the same kind on `config`, solved: OpenCMP's ``solver.reset_model(); solver.solve()``."""
    s = type(solver)(type(solver.model), config)
    s.solve()
    return s


def h_rates(n_elements: Sequence[int], errors: Sequence[float], dim: int) -> List[float]:
    """OpenCMP's h-convergence rates (error_analysis.py:102-105)."""
    return [math.log(errors[n] / errors[n + 1]) / math.log(n_elements[n + 1] / (n_elements[n] * 2.0 ** (dim - 1)))
            for n in range(len(errors) - 1)]


def p_rates(n_dofs: Sequence[int], errors: Sequence[float]) -> List[float]:
    """OpenCMP's p-convergence rates (error_analysis.py:155-157)."""
    return [math.log(errors[n] / errors[n + 1]) / math.log(n_dofs[n + 1] / n_dofs[n]) for n in range(len(errors) - 1)]


def format_table(rows: List[list], floatfmt: Sequence[str]) -> str:
    """The convergence table: ``tabulate`` with OpenCMP's headers and formats when it is installed,
    otherwise plain columns with the same formats."""
    try:
        import tabulate
        return tabulate.tabulate(rows, headers='firstrow', floatfmt=tuple(floatfmt))
    except ImportError:
        pass
    head, body = rows[0], rows[1:]

    def cell(v, f):
        if isinstance(v, float):
            return format(v, f)
        if isinstance(v, int) and f.endswith('f'):
            return format(float(v), f)
        return str(v)
    cells = [[cell(v, floatfmt[i]) for i, v in enumerate(r)] for r in body]
    w = [max([len(str(head[i]))] + [len(r[i]) for r in cells]) for i in range(len(head))]
    lines = ['  '.join(str(h).rjust(w[i]) for i, h in enumerate(head)),
             '  '.join('-' * w[i] for i in range(len(head)))]
    lines += ['  '.join(c.rjust(w[i]) for i, c in enumerate(r)) for r in cells]
    return '\n'.join(lines)


def h_convergence(config_parser: ConfigParser, solver, sol, var: str) -> None:
    """Re-solve on uniformly refined meshes and print the errors and rates
    (error_analysis.py:53-108)."""
    _check_average(config_parser, var)
    num = config_parser.get_item(['ERROR ANALYSIS', 'num_refinements'], int)
    model = solver.model
    n_el = [model.mesh.ne]
    errs = [model.l2_error_of(var, solver.t)]
    mesh = model.mesh
    for n in range(num):
        mesh = refine_uniform(mesh)
        cfg = ConfigParser.from_parser(config_parser)
        cfg.refined_mesh = mesh
        s = _resolve(solver, cfg)
        err = s.model.l2_error_of(var, s.t)
        n_el.append(mesh.ne)
        errs.append(err)
        print('L2 norm at refinement {0}: {1}'.format(n + 1, err))
        del s
    rates = h_rates(n_el, errs, model.mesh.dim)
    rows = [['Refinement Level', 'Mesh Elements', 'Error', 'Convergence Rate'], [1, n_el[0], errs[0], 0]]
    for n in range(num):
        rows.append(['1/{}'.format(int(2 ** (n + 1))), n_el[n + 1], errs[n + 1], rates[n]])
    print(format_table(rows, ('.1f', '.1f', '.3e', '.2f')))


def p_convergence(config_parser: ConfigParser, solver, sol, var: str) -> None:
    """Re-solve with the interpolant order raised by one each time and print the errors and rates
    (error_analysis.py:111-160). The spaces here go up to order 3."""
    _check_average(config_parser, var)
    num = config_parser.get_item(['ERROR ANALYSIS', 'num_refinements'], int)
    model = solver.model
    if var not in getattr(model, 'vars', {}):
        raise NotImplementedError('p-convergence of {} is not on the GPU path for this model'.format(var))
    order = model.interp_ord
    if order + num > 3:
        raise NotImplementedError('p-convergence to order {}: the GPU spaces go up to order 3'.format(order + num))
    n_dofs = [model.vars[var].space.ndof]
    orders = [order]
    errs = [model.l2_error_of(var, solver.t)]
    for n in range(num):
        cfg = ConfigParser.from_parser(config_parser)
        cfg['FINITE ELEMENT SPACE']['interpolant_order'] = str(order + n + 1)
        s = _resolve(solver, cfg)
        err = s.model.l2_error_of(var, s.t)
        n_dofs.append(s.model.vars[var].space.ndof)
        orders.append(order + n + 1)
        errs.append(err)
        print('L2 norm at refinement {0}: {1}'.format(n + 1, err))
        del s
    rates = p_rates(n_dofs, errs)
    rows = [['Interpolant Order', 'DOFs', 'Error', 'Convergence Rate'], [orders[0], n_dofs[0], errs[0], 0]]
    for n in range(num):
        rows.append([orders[n + 1], n_dofs[n + 1], errs[n + 1], rates[n]])
    print(format_table(rows, ('.1f', '.1f', '.3e', '.2f')))
