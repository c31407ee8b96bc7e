"""Host helpers of bench.py on the CPU: the summary of the nvidia-smi clock
samples taken during the timed region (median SM clock, maximum, the
throttle reasons seen), and the thread that clears the end-to-end loop's
idle host box."""
import importlib.util
import pathlib
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parents[1]


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _row(sm, mx, hw="Not Active", hwt="Not Active", swt="Not Active", pcap="Not Active"):
    # --query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,
    # hw_slowdown,hw_thermal_slowdown,sw_thermal_slowdown,sw_power_cap (csv,noheader,nounits)
    return ["0", str(sm), str(mx), "612.50", "0x0000000000000000", hw, hwt, swt, pcap]


def test_clock_summary():
    b = _bench()
    c = b.Clocks(0)
    assert c.summary()["reasons"] == ["unsampled"]
    c.rows = [_row(2070, 2070), _row(2055, 2070, pcap="Active"), _row(2070, 2070), ["garbled"]]
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"] and s["samples"] == 4
    c.rows = [_row(1410, 2070, hwt="Active"), _row(1395, 2070, hw="Active", swt="Active")]
    s = c.summary()
    assert s["sm_mhz"] == 1402.5
    assert s["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"]


def test_box_clearer_clears_the_idle_box_between_calls():
    b = _bench()
    boxes = [np.ones(1 << 16), np.ones(1 << 16)]
    clearer = b.BoxClearer(0.001)
    seen = []
    for q in range(6):
        clearer.wait()
        if q >= 1 and q + 1 < 6:
            clearer.clear(boxes[(q + 1) % 2])
        seen.append(float(boxes[q % 2].sum()))
        boxes[q % 2][:] = 1.0  # the call writes its solution into the box
        time.sleep(0.005)
    clearer.close()
    # steps 0 and 1 find the boxes as given; every later step finds its box
    # cleared by the thread while the step before it ran
    assert seen == [float(1 << 16)] * 2 + [0.0] * 4
    assert not clearer.thread.is_alive()
