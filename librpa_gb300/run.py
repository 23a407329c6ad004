"""One RPA correlation-energy evaluation of a synthetic workload, through the C API.

    python -m librpa_gb300.run --workload fcc16_k333 --chi0 bf16x3 --ec chol [--repeat N]

Loads the workload with the librpa_set_* setters, makes ``--repeat`` calls of
librpa_get_rpa_correlation_energy (the call ``task=rpa`` of the reference driver makes,
driver/task/rpa.cpp:30) and prints one JSON line per call with E_c and the stage times.
This is the command the kernel profiles are captured with.  A batch workload (a list of
independent systems, synthetic.BATCHES) is loaded into one handler per system and every
repeat evaluates them all, one call each (or, with ``--concurrent``, one batch call that runs them
concurrently); its line reports the summed wall time and the per-system energies.
"""
import argparse
import json
import time

from . import load_system, n_ibz, rpa_correlation_energy_batch, Handler, Options, gb300_options, Minimax, LIBRI, EC_CHOL, EC_CHOL_FP64, EC_LU_FP64
from . import synthetic

CHI0 = {"fp64": 0, "bf16x3": 1, "fp32": 2}
EC = {"lu": EC_LU_FP64, "chol": EC_CHOL, "chol64": EC_CHOL_FP64}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="fcc16_k333", choices=sorted(synthetic.WORKLOADS) + sorted(synthetic.BATCHES))
    ap.add_argument("--chi0", default="bf16x3", choices=list(CHI0))
    ap.add_argument("--ec", default="chol", choices=list(EC))
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--threads", type=int, default=0, help="host threads of the concurrent batch call (0: up to 4)")
    ap.add_argument("--concurrent", action="store_true",
                    help="batch workloads: one librpa_gb300_get_rpa_correlation_energy_batch call for all systems")
    a = ap.parse_args(argv)
    if a.workload in synthetic.BATCHES:
        return run_batch(a)
    s = synthetic.WORKLOADS[a.workload]()
    h = Handler()
    load_system(h, s)
    o = Options(nfreq=s.nfreq, tfgrids_type=Minimax, parallel_routing=LIBRI, minimax_emin=s.minimax_emin,
                minimax_emax=s.minimax_emax)
    h.set_gb300_options(gb300_options(chi0_precision=CHI0[a.chi0], ec_path=EC[a.ec]))
    for _ in range(a.repeat):
        t = time.time()
        ec, _ = h.get_rpa_correlation_energy(o, n_ibz(s))
        dt = time.time() - t
        st = h.stats()
        print(json.dumps({"workload": a.workload, "chi0": a.chi0, "ec_path": a.ec, "ec": ec, "wall_s": dt,
                          **{k: st[k] for k in ("t_gf", "t_chi0", "t_ftct", "t_ec", "chi0_flops", "ec_flops",
                                                "n_launches")}}), flush=True)


def run_batch(a):
    systems = synthetic.BATCHES[a.workload]()
    hs = []
    for s in systems:
        h = Handler()
        load_system(h, s)
        h.set_gb300_options(gb300_options(chi0_precision=CHI0[a.chi0], ec_path=EC[a.ec]))
        o = Options(nfreq=s.nfreq, tfgrids_type=Minimax, parallel_routing=LIBRI, minimax_emin=s.minimax_emin,
                    minimax_emax=s.minimax_emax)
        hs.append((h, o, s))
    for _ in range(a.repeat):
        t = time.time()
        if a.concurrent:
            ecs = list(rpa_correlation_energy_batch([h for h, _, _ in hs], [o for _, o, _ in hs], a.threads))
        else:
            ecs = [h.get_rpa_correlation_energy(o, n_ibz(s))[0] for h, o, s in hs]
        dt = time.time() - t
        print(json.dumps({"workload": a.workload, "chi0": a.chi0, "ec_path": a.ec, "systems": len(hs),
                          "concurrent": a.concurrent, "atoms": [s.n_atoms for _, _, s in hs], "ec": ecs,
                          "wall_s": dt}), flush=True)


if __name__ == "__main__":
    main()
