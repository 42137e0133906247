"""Solution files and restart on the GPU path: opencmp/helpers/saving.py:24-93 (SolutionFileSaver)
and the checkpoint selection of opencmp/solvers/base_solver.py:91-213.

Files are written where OpenCMP writes them, ``<run_dir>/output/<model>_sol/<model>_<t>.sol``, with
``<t>`` formatted by ``str(float)`` as OpenCMP does. NGSolve's own ``GridFunction.Save`` format is not
available here; the content is this library's: the magic ``OCMPSOL1``, the number of variables, and
for each variable its name, its number of dofs and its FP64 values in the space's dof order. A
restart reads the same format back as the initial condition.
"""
from __future__ import annotations

import logging
import math
import os
import struct
from pathlib import Path
from typing import Dict, List, Tuple

import numpy as np

MAGIC = b'OCMPSOL1'


def write_sol(path: str, state: Dict[str, np.ndarray]) -> None:
    """Write the named FP64 vectors to one solution file (written to a temporary name, then moved)."""
    tmp = str(path) + '.tmp'
    with open(tmp, 'wb') as fh:
        fh.write(MAGIC)
        fh.write(struct.pack('<I', len(state)))
        for name, vec in state.items():
            b = name.encode('utf-8')
            v = np.ascontiguousarray(vec, dtype='<f8')
            fh.write(struct.pack('<I', len(b)))
            fh.write(b)
            fh.write(struct.pack('<Q', v.size))
            fh.write(v.tobytes())
    os.replace(tmp, path)


def read_sol(path: str) -> Dict[str, np.ndarray]:
    """The named FP64 vectors of a solution file written by :func:`write_sol`."""
    with open(path, 'rb') as fh:
        if fh.read(8) != MAGIC:
            raise ValueError('{} is not a solution file of this library (magic {!r} expected)'.format(path, MAGIC))
        (nv,) = struct.unpack('<I', fh.read(4))
        out = {}
        for _ in range(nv):
            (nb,) = struct.unpack('<I', fh.read(4))
            name = fh.read(nb).decode('utf-8')
            (n,) = struct.unpack('<Q', fh.read(8))
            data = fh.read(8 * n)
            if len(data) != 8 * n:
                raise ValueError('{}: truncated solution file'.format(path))
            out[name] = np.frombuffer(data, dtype='<f8').copy()
    return out


class SolutionFileSaver:
    """Writes the model's state after the accepted steps the save frequency selects
    (``[VISUALIZATION] save_frequency = <k>, numit | time``)."""

    def __init__(self, model, config):
        save_type = config.get_item(['VISUALIZATION', 'save_type'], str, quiet=True)
        if save_type not in ('.sol', '.vtu'):
            print("Can't output to file type {}.".format(save_type))
        if save_type == '.vtu':
            raise NotImplementedError('.vtu output is not on the GPU path (save_type = .sol)')
        run_dir = config.get_item(['OTHER', 'run_dir'], str)
        self.model = model
        self.save_dir_sol = os.path.join(run_dir, 'output', model.name() + '_sol')
        Path(self.save_dir_sol).mkdir(parents=True, exist_ok=True)
        freq = config.get_list(['VISUALIZATION', 'save_frequency'], str, quiet=True)
        self.freq = (float(freq[0]), freq[1].strip())
        if self.freq[1] not in ('time', 'numit'):
            raise ValueError('Save frequency must be specified either per amount of time ("time") or per number of '
                             'iterations ("numit").')

    def filename(self, t: float) -> str:
        return os.path.join(self.save_dir_sol, '{}_{}.sol'.format(self.model.name(), str(t)))

    def save(self, t: float) -> None:
        write_sol(self.filename(t), self.model.state())

    def after_step(self, num_iters: int, t: float, t0: float, dt: float) -> None:
        """The save test of base_solver.py:562-586 after an accepted step."""
        k, kind = self.freq
        if kind == 'numit':
            if num_iters % int(k) == 0:
                self.save(t)
            return
        if k < 1.0:
            tmp = (t - t0) * (1.0 / k)
            tmp = tmp - 1.0 if tmp < 1.0 else tmp % 1.0
        else:
            tmp = (t - t0) % k
        if math.isclose(tmp, 0.0, abs_tol=dt * 1e-2):
            self.save(t)


def checkpoint_time(checkpoint: Path, model_name: str) -> float:
    """The time encoded in a checkpoint name ``<model>_<t>.sol`` (base_solver.py:91-112)."""
    prefix = model_name + '_'
    if not checkpoint.name.startswith(prefix) or checkpoint.suffix != '.sol':
        raise ValueError('Restart checkpoint "{}" must be named "{}<time>.sol" for the active model.'
                         .format(checkpoint, prefix))
    text = checkpoint.name[len(prefix):-len(checkpoint.suffix)]
    try:
        t = float(text)
    except ValueError:
        raise ValueError('Could not determine the restart time from checkpoint "{}". Expected the filename format '
                         '"{}<time>.sol".'.format(checkpoint, prefix))
    if not math.isfinite(t):
        raise ValueError('Restart checkpoint "{}" does not contain a finite time.'.format(checkpoint))
    return t


def select_checkpoint(restart_from: str, run_dir: Path, model_name: str) -> Tuple[Path, float]:
    """An explicit checkpoint (absolute, or relative to the run directory) or, for ``LATEST``, the
    latest valid checkpoint of this model (base_solver.py:114-144)."""
    if restart_from.upper() == 'LATEST':
        out = run_dir / 'output' / (model_name + '_sol')
        found: List[Tuple[float, Path]] = []
        if out.exists():
            for f in out.rglob(model_name + '_*.sol'):
                try:
                    found.append((checkpoint_time(f, model_name), f.resolve()))
                except ValueError:
                    continue
        if not found:
            raise FileNotFoundError('No valid .sol checkpoint for model "{}" was found in "{}". Set '
                                    'resume_from_previous to False to start a new simulation.'.format(model_name, out))
        t, f = max(found, key=lambda item: item[0])
        return f, t
    f = Path(restart_from).expanduser()
    if not f.is_absolute():
        f = run_dir / f
    f = f.resolve()
    if not f.is_file():
        raise FileNotFoundError('The restart checkpoint "{}" does not exist.'.format(f))
    return f, checkpoint_time(f, model_name)


def resolve_restart(config, model_name: str, history_order: int):
    """Checkpoint handling of Solver.__init__ (base_solver.py:150-213): returns the checkpoint path
    (or None) and moves the start of time_range to its time. Multistep schemes are refused, since a
    single saved solution cannot restore their history."""
    resume = config.get_item(['OTHER', 'resume_from_previous'], bool)
    restart_from = config.get_item(['OTHER', 'restart_from'], str, quiet=True).strip()
    if restart_from and not resume:
        raise ValueError('restart_from is set to "{}", but resume_from_previous is False. Enable '
                         'resume_from_previous or remove restart_from.'.format(restart_from))
    if not resume:
        return None
    scheme = config.get_item(['TRANSIENT', 'scheme'], str)
    if history_order > 1:
        raise NotImplementedError('resume_from_previous only supports single-step time discretization schemes. The '
                                  '"{}" scheme needs {} previous time steps, which cannot be recovered from the saved '
                                  '.sol files since save_frequency may skip time steps.'.format(scheme, history_order))
    if not restart_from:
        restart_from = 'LATEST'
        logging.warning('resume_from_previous without restart_from is deprecated and currently means restart_from = '
                        'LATEST. Set restart_from explicitly in the [OTHER] section.')
    run_dir = Path(config.get_item(['OTHER', 'run_dir'], str)).resolve()
    path, t_restart = select_checkpoint(restart_from, run_dir, model_name)
    config.set('OTHER', 'restart_from', str(path))
    tr = [s.strip() for s in config.get('TRANSIENT', 'time_range').split(',')]
    t_end = float(tr[-1])
    if t_restart >= t_end or math.isclose(t_restart, t_end, rel_tol=1e-9):
        print('Simulation is already complete at t = {}, the end of time_range. Nothing to resume.'.format(t_restart))
        raise SystemExit(0)
    tr[0] = str(t_restart)
    config.set('TRANSIENT', 'time_range', ', '.join(tr))
    print('Resuming from checkpoint: {}'.format(path))
    return path
