"""CPU oracle for the OSEM hot path — TEST INFRASTRUCTURE ONLY.

A restatement in numpy (float64 by default, float32 on request) of the reference's
algorithms, each function citing the reference file:line it follows. Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline / reference arm may import it,
and only as the checker or the timed CPU baseline; the product path never calls it.

Parity pin: tests/golden/*.npz hold outputs of the reference's own functions, run
on CPU in this repository's build container by tests/golden/make_golden.py on
seeded synthetic inputs; tests/test_oracle_golden.py checks this oracle against them.
"""
