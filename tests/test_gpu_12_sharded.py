"""The sharded ensemble forms on the GPU, with the shares run one after the
other in one process (every call of this suite has one GPU): each share of
the 256-chain ensemble run as its own Batch (ensemble.batch_compute, the
per-rank compute of shard.run_sharded) gives every chain's counts and final
configuration exactly as that chain run alone; each share of a request
stream served by its own Server (ensemble.stream_compute) gives every
request's result exactly as one server holding the whole stream."""
import dataclasses

import pytest

from dym_symanzik_action_gb300 import ensemble, shard, tables
from dym_symanzik_action_gb300.workloads import ensemble as ens_specs
from dym_symanzik_action_gb300.workloads import llr_requests

pytestmark = pytest.mark.gpu


def test_sharded_batches_equal_chains_alone(engine):
    specs = [s for s in ens_specs() if s.Nx <= 12][:10] + [s for s in ens_specs() if s.group == "BI"][:4]
    sweeps, nhit = 2, 10
    work = shard.chain_work([s.links for s in specs], sweeps)
    merged = {}
    for rank in range(2):  # the two ranks' shares, in turn
        share = shard.partition(work, 2)[rank]
        merged.update(ensemble.batch_compute(specs, sweeps, nhit, 0, autotune=False)(share))
    assert sorted(merged) == list(range(len(specs)))
    groups = {}
    for i, s in enumerate(specs):
        g = groups.setdefault(s.group, engine.load_group(tables.ensure_table(s.group)))
        lat = engine.Lattice(g, 4, s.Nt, s.Nx, *s.beta, s.seed, start=s.start)
        st = lat.update(sweeps, nhit)
        assert merged[i] == [st.hits, st.accepts, ensemble.links_digest(lat.links)], i
        lat.close()


def test_sharded_stream_equals_one_server(engine):
    reqs = [dataclasses.replace(r, K=4, NRM=3, arrival=0.0) for r in llr_requests(n=40) if r.Nx <= 8][:8]
    work = [float(r.nplaq * r.K * r.NRM) for r in reqs]
    one = ensemble.stream_compute(reqs, 0, nhit=10, step_sweeps=4)(list(range(len(reqs))))
    merged = {}
    for rank in range(2):
        merged.update(ensemble.stream_compute(reqs, 0, nhit=10, step_sweeps=4)(shard.partition(work, 2)[rank]))
    assert sorted(merged) == sorted(one)
    for rid in one:
        assert merged[rid][:3] == one[rid][:3], rid  # status, a, sweeps (latencies differ)
