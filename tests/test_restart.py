"""Solution files and restart (opencmp/helpers/saving.py:24-93, opencmp/solvers/base_solver.py:91-213).

The CPU tests cover the file format and the checkpoint selection; the GPU test follows the
reference's restart test (pytests/full_system/restart/test_restart.py:76-133) on its own run
directory: solve 0 -> 0.1 with implicit Euler saving every step, throw away the files after
t = 0.05, resume through run() with each way of naming the checkpoint, and compare the final
solutions: ||u_resumed - u_uninterrupted||_L2 / ||u_uninterrupted||_L2 < 1e-10.
"""
import logging
import os
import shutil
from pathlib import Path

import numpy as np
import pytest

from opencmp_gb300 import saving
from opencmp_gb300.config import ConfigParser

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIX = os.path.join(ROOT, 'tests', 'golden', 'fixtures', 'restart_transient_poisson')
MESH = os.path.join(ROOT, 'tests', 'golden', 'unit_square_coarse.npz')
T_RESTART, T_FINAL = 0.05, 0.1


def _case(tmp_path: Path) -> Path:
    case = tmp_path / 'transient_poisson'
    shutil.copytree(FIX, case)
    cfg = case / 'config'
    text = cfg.read_text().replace('run_dir = .', 'run_dir = ' + str(case))
    text = text.replace('filename = pytests/mesh_files/unit_square_coarse.vol', 'filename = ' + MESH)
    cfg.write_text(text)
    return case


def _sol_time(f: Path) -> float:
    return float(f.stem.split('_')[1])


def _sol_files(d: Path):
    return sorted(d.glob('poisson_*.sol'), key=_sol_time)


def test_solution_file_round_trip(tmp_path):
    st = {'u': np.linspace(0, 1, 17), 'p': np.array([3.5, -1e-300, np.pi])}
    f = tmp_path / 'poisson_0.05.sol'
    saving.write_sol(str(f), st)
    back = saving.read_sol(str(f))
    assert list(back) == ['u', 'p'] and all(np.array_equal(back[k], st[k]) for k in st)
    (tmp_path / 'bad.sol').write_bytes(b'NGSOLVE!')
    with pytest.raises(ValueError):
        saving.read_sol(str(tmp_path / 'bad.sol'))


def test_checkpoint_names_and_selection(tmp_path):
    d = tmp_path / 'output' / 'poisson_sol'
    d.mkdir(parents=True)
    for t in (0.0, 0.01, 0.09999999999999999, 0.05):
        saving.write_sol(str(d / 'poisson_{}.sol'.format(t)), {'u': np.zeros(2)})
    (d / 'poisson_notatime.sol').write_bytes(b'x')
    (d / 'mcpoisson_999.0.sol').write_bytes(b'x')          # another model's checkpoint
    f, t = saving.select_checkpoint('LATEST', tmp_path, 'poisson')
    assert t == 0.09999999999999999 and f.name == 'poisson_0.09999999999999999.sol'
    f, t = saving.select_checkpoint('output/poisson_sol/poisson_0.05.sol', tmp_path, 'poisson')
    assert t == 0.05 and f.is_absolute()
    f2, _ = saving.select_checkpoint(str(f), tmp_path, 'poisson')
    assert f2 == f
    with pytest.raises(FileNotFoundError):
        saving.select_checkpoint('output/poisson_sol/poisson_0.5.sol', tmp_path, 'poisson')
    with pytest.raises(FileNotFoundError):
        saving.select_checkpoint('LATEST', tmp_path, 'ins')
    with pytest.raises(ValueError):
        saving.checkpoint_time(Path('poisson_inf.sol'), 'poisson')
    with pytest.raises(ValueError):
        saving.checkpoint_time(Path('ins_0.1.sol'), 'poisson')


def test_resolve_restart_rules(tmp_path, caplog):
    case = _case(tmp_path)
    d = case / 'output' / 'poisson_sol'
    d.mkdir(parents=True)
    saving.write_sol(str(d / 'poisson_0.05.sol'), {'u': np.zeros(2)})
    c = ConfigParser(str(case / 'config'))
    assert saving.resolve_restart(c, 'poisson', 1) is None
    c['OTHER']['restart_from'] = 'LATEST'
    with pytest.raises(ValueError, match='resume_from_previous is False'):
        saving.resolve_restart(c, 'poisson', 1)
    c = ConfigParser(str(case / 'config'))
    c['OTHER']['resume_from_previous'] = 'True'
    with pytest.raises(NotImplementedError, match='single-step'):
        saving.resolve_restart(c, 'poisson', 2)
    with caplog.at_level(logging.WARNING):
        f = saving.resolve_restart(c, 'poisson', 1)
    assert 'without restart_from is deprecated' in caplog.text
    assert f.name == 'poisson_0.05.sol' and float(c.get('TRANSIENT', 'time_range').split(',')[0]) == 0.05
    c = ConfigParser(str(case / 'config'))
    c['OTHER']['resume_from_previous'] = 'True'
    c['OTHER']['restart_from'] = 'LATEST'
    saving.write_sol(str(d / 'poisson_0.1.sol'), {'u': np.zeros(2)})
    with pytest.raises(SystemExit):
        saving.resolve_restart(c, 'poisson', 1)


@pytest.mark.gpu
@pytest.mark.parametrize('restart_selector', ['relative', 'absolute', 'LATEST', 'legacy'])
def test_resume_matches_uninterrupted_solve(gpu_lib, tmp_path, restart_selector, caplog):
    import torch
    from opencmp_gb300.run import run
    case = _case(tmp_path)
    sol_dir = case / 'output' / 'poisson_sol'
    solver, sol = run(str(case / 'config'))
    saved = _sol_files(sol_dir)
    assert _sol_time(saved[0]) == 0.0 and _sol_time(saved[-1]) == pytest.approx(T_FINAL)
    reference = tmp_path / 'reference_final.sol'
    shutil.copy(saved[-1], reference)
    space = sol['u'].space
    for f in saved:
        if _sol_time(f) > T_RESTART:
            f.unlink()
    restart_from = _sol_files(sol_dir)[-1]
    assert _sol_time(restart_from) == pytest.approx(T_RESTART)
    if restart_selector == 'LATEST':
        shutil.copy(restart_from, sol_dir / 'mcpoisson_999.0.sol')
    cfg = case / 'config'
    text = cfg.read_text().replace('resume_from_previous = False', 'resume_from_previous = True')
    if restart_selector == 'relative':
        text += '\nrestart_from = output/poisson_sol/' + restart_from.name + '\n'
    elif restart_selector == 'absolute':
        text += '\nrestart_from = ' + str(restart_from.resolve()) + '\n'
    elif restart_selector == 'LATEST':
        text += '\nrestart_from = LATEST\n'
    cfg.write_text(text)
    with caplog.at_level(logging.WARNING):
        run(str(cfg))
    if restart_selector == 'legacy':
        assert 'without restart_from is deprecated' in caplog.text
    resumed = _sol_files(sol_dir)[-1]
    assert _sol_time(resumed) == pytest.approx(T_FINAL)
    expected = torch.as_tensor(saving.read_sol(str(reference))['u'], device='cuda')
    got = torch.as_tensor(saving.read_sol(str(resumed))['u'], device='cuda')
    err = space.l2_error(expected - got)
    norm = space.l2_error(expected)
    assert norm > 0.0
    assert err / norm < 1e-10, err / norm
