"""CPU oracle for the MoL finite-difference evolution path.

TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline leg may import, call or link anything under
oracle/; the product (nrpytutorial_gb300/, libnrgpu.so) never does.

Contents: a numpy (FP64) restatement of the reference's algorithms, each
function citing the zachetienne/nrpytutorial file:line it follows, and
gen_ref.py, which runs the reference's own code generator (when the reference
checkout is available) to build oracle/_ref/ -- the reference-generated C
kernels compiled with gcc -- and the golden fixtures in tests/golden/.

Parity pinning: the numpy restatement is checked against (1) the
reference's trusted-value unit tests (*/tests/trusted_values_dict.py,
md5-seeded inputs, 30-digit expected values), (2) the SENR curvilinear-BC
golden files, and (3) outputs of the reference-generated C on seeded grids
(tests/golden/*.npz, made by oracle/gen_ref.py).
"""
