"""Host-side pieces of bench.py (CPU): the clock-sample summary that goes into the bench line's
``clocks`` object, and the roofline peak it divides by."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def test_clock_samples_summary():
    import bench
    c = bench.Clocks.__new__(bench.Clocks)
    c.proc = None
    # nvidia-smi rows: clocks.sm, clocks.max.sm, hw_slowdown, hw_thermal_slowdown, sw_thermal_slowdown,
    # sw_power_cap (csv, no header, no units)
    c.samples = [['2070', '2070', 'Not Active', 'Not Active', 'Not Active', 'Active'],
                 ['1980', '2070', 'Not Active', 'Active', 'Not Active', 'Not Active'],
                 ['2040', '2070', 'Not Active', 'Not Active', 'Not Active', 'Not Active'],
                 ['[N/A]', '[N/A]', '[N/A]', '[N/A]', '[N/A]', '[N/A]'],
                 []]
    s = c.stop()
    assert s['sm_mhz'] == 2040.0 and s['sm_max_mhz'] == 2070.0 and s['samples'] == 3
    assert s['reasons'] == ['hw_thermal_slowdown', 'sw_power_cap']
    c.samples = []
    s = c.stop()
    assert s['sm_mhz'] is None and s['sm_max_mhz'] is None and s['reasons'] == [] and s['samples'] == 0


def test_roofline_peak_is_the_measured_copy_bandwidth():
    import bench
    peak, kind = bench.peaks()
    path = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    if os.path.isfile(path):
        with open(path) as fh:
            assert (peak, kind) == (float(json.load(fh)['hbm_gbs']), 'measured')
    else:
        assert (peak, kind) == (6800.0, 'fallback')
