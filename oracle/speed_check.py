"""Transport speed of the oracle port against the upstream code compiled
unmodified (oracle/_ref, make -C oracle ref), on one deck, on the same host
with the same thread count.  Test infrastructure: it backs the use of the
port as the CPU baseline where the upstream build cannot run (the GPU host
has no upstream checkout).  Both time only replicated_transport's history
branch (the upstream transport timer): the harness around
replicated_transport<std::vector<Photon>>, the port around bo_transport plus
bo_post_process.

    python oracle/speed_check.py [--side 50] [--photons 1e6] [--steps 2]
                                 [--threads N] [--repeats 3]

Prints one JSON line: histories/s of each per repeat, and their ratio.
Needs the upstream sources at $BRANSON_REFERENCE (default /root/reference).
"""
import argparse
import json
import os
import re
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--side", type=int, default=50)
    p.add_argument("--photons", type=float, default=1e6)
    p.add_argument("--steps", type=int, default=2)
    p.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    p.add_argument("--repeats", type=int, default=3)
    a = p.parse_args()
    import subprocess
    import oracle as O
    from branson_gb300 import deck as D

    ref = os.environ.get("BRANSON_REFERENCE", "/root/reference")
    subprocess.run(["make", "-s", "-C", HERE, "ref", "port", f"REF={ref}"], check=True)
    dk = D.hot_zone(n_per_axis=a.side, photons=int(a.photons), n_steps=10)
    up, port = [], []
    for _ in range(a.repeats):
        with tempfile.TemporaryDirectory() as out:
            txt = O.run_reference_harness(dk, out, a.steps, n_threads=a.threads, dump=False)
        m = re.search(r"HARNESS histories (\d+) transport_s ([0-9.eE+-]+)", txt)
        up.append(int(m.group(1)) / float(m.group(2)))
        orc = O.Oracle(dk, n_threads=a.threads)
        h = s = 0
        for _ in range(a.steps):
            r = orc.step()
            h += len(r.source)
            s += r.transport_s
        port.append(h / s)
    best_up, best_port = max(up), max(port)
    print(json.dumps({"deck": f"hot_zone {a.side}^3", "photons_per_step": int(a.photons), "steps": a.steps,
                      "threads": a.threads, "upstream_hist_per_s": up, "port_hist_per_s": port,
                      "port_over_upstream_best": best_port / best_up}))


if __name__ == "__main__":
    main()
