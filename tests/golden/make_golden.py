"""Regenerate the golden vectors under tests/golden/ from the reference fixtures.

Reads ``tests/testthat/Group1/data/lba_data{0..6}.rda`` of the reference
checkout (R serialisation, decoded by ggdmc_gb300.rda) and writes one compact
``lba_fx{N}.npz`` per fixture.  Each holds the flattened design, the trials of
the single-subject DMI and of the hierarchical DMIs, the priors, and the first
stored MCMC slice of ``sub_samples`` and ``pop_samples``: theta, summed log
prior and log-likelihood per chain.  Those stored values were computed by the
reference's own likelihood and prior packages (ggdmcLikelihood, ggdmcPrior)
when the fixture generators (``tests/testthat/Group1/data/*_lba_*.r``) ran, so
they are known answers for the per-subject LBA log-likelihood sum, the
truncated-normal / uniform log priors and the hyper log-likelihood.

Usage (needs the reference checkout, given as an argument or by the
GGDMC_REFERENCE environment variable; the GPU machine does not):
    python tests/golden/make_golden.py [REFERENCE_ROOT]
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from ggdmc_gb300.rda import load_rda  # noqa: E402
from ggdmc_gb300.dmi import (SubjectBatch, model_from_dmi, prior_table,  # noqa: E402
                             subject_from_dmi)

# Hierarchical subjects kept per fixture (all 32 for fixture 6, the design of
# the 32-subject hierarchical workload; a prefix elsewhere keeps files small).
KEEP_SUBJECTS = {6: 32}
DEFAULT_KEEP = 8


def _slice(post):
    th = post["theta"].array()                    # [P, C, nmc]
    ll = post["log_likelihoods"].array()          # [C, nmc]
    lp = post["summed_log_prior"].array()
    return (np.ascontiguousarray(th[:, :, 0].T), np.ascontiguousarray(ll[:, 0]),
            np.ascontiguousarray(lp[:, 0]))


def build(ref_root: str, fx: int) -> dict:
    d = load_rda(os.path.join(ref_root, "tests/testthat/Group1/data", f"lba_data{fx}.rda"))
    sub_dmi = d["sub_dmis"][0]
    model = model_from_dmi(sub_dmi)
    out = {
        "pnames": np.array(model.pnames),
        "accumulators": np.array(model.accumulators),
        "cell_names": np.array(model.cell_names),
        "const_names": np.array(model.const_names),
        "constants": model.constants,
        "param_src": model.param_src,
        "resp": model.resp,
    }
    sub = subject_from_dmi(sub_dmi, model, "sub")
    out["sub_rt"], out["sub_cell"] = sub.rt, sub.cell
    out["sub_theta"], out["sub_ll"], out["sub_lp"] = _slice(d["sub_samples"])
    out["sub_prior"] = prior_table(d["sub_priors"]["p_prior"])

    pop = d["pop_samples"]
    phi_th, phi_ll, phi_lp = _slice(pop["phi"])
    out["phi_theta"], out["phi_ll"], out["phi_lp"] = phi_th, phi_ll, phi_lp
    sts = pop["subject_theta"]
    ths, lls, lps = zip(*[_slice(p) for p in sts.items])
    out["subj_theta"] = np.stack(ths)             # [S, C, P] (all subjects)
    out["subj_ll"] = np.stack(lls)
    out["subj_lp"] = np.stack(lps)
    out["pop_p_prior"] = prior_table(d["pop_priors"]["p_prior"])
    out["pop_h_prior"] = prior_table(d["pop_priors"]["h_prior"])

    keep = KEEP_SUBJECTS.get(fx, DEFAULT_KEEP)
    dm = d["pop_dmis"]
    subs = [subject_from_dmi(dm[i], model_from_dmi(dm[i]), str(i)) for i in range(keep)]
    batch = SubjectBatch.pack(subs)
    out["pop_rt"], out["pop_cell"], out["pop_offsets"] = batch.rt, batch.cell, batch.offsets
    return out


def raw_dmi(ref_root: str, fx: int) -> dict:
    """The single-subject DMI, its priors and its samples' shape as the S4
    slots hold them (before flattening): what a .Call shim reads with the R
    C API and hands to the converters of include/ggdmc_dmi.h."""
    d = load_rda(os.path.join(ref_root, "tests/testthat/Group1/data", f"lba_data{fx}.rda"))
    dmi = d["sub_dmis"][0]
    m = dmi["model"]
    mb = m["model_boolean"]
    consts = m["constants"]
    data = dmi["data"]
    prior = d["sub_priors"]["p_prior"]
    fields = [list(item.names) for item in prior.items]
    values = [[float(v.data[0]) if len(v.data) else np.nan for v in item.items] for item in prior.items]
    return {
        "type": np.array(m["type"].data),
        "model_boolean": np.asarray(mb.data, np.int32),          # column-major [ncell, npxc, K]
        "model_boolean_dim": np.asarray(mb.attrs["dim"].data, np.int32),
        "pxc_names": np.array(m["parameter_x_condition_names"].data),
        "pnames": np.array(m["pnames"].data),
        "constants": np.asarray(consts.data, np.float64),
        "const_names": np.array(consts.attrs["names"].data),
        "cell_names": np.array(m["cell_names"].data),
        "accumulators": np.array(m["accumulators"].data),
        "data_names": np.array(data.names),
        "data_len": np.array([len(v.data) for v in data.items], np.int32),
        "data_rt": np.concatenate([np.asarray(v.data, np.float64) for v in data.items]),
        "prior_fields": np.array(fields),
        "prior_values": np.array(values, np.float64),
    }


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GGDMC_REFERENCE")
    if not ref:
        sys.exit("usage: make_golden.py REFERENCE_ROOT (or set GGDMC_REFERENCE)")
    for fx in range(7):
        arrs = build(ref, fx)
        path = os.path.join(HERE, f"lba_fx{fx}.npz")
        np.savez_compressed(path, **arrs)
        print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB)")
    for fx in (3, 6):
        path = os.path.join(HERE, f"dmi_raw_fx{fx}.npz")
        np.savez_compressed(path, **raw_dmi(ref, fx))
        print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB)")


if __name__ == "__main__":
    main()
