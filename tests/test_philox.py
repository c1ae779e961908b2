"""CPU: the Philox4x32-10 generator (device header and the oracle's restatement)
against the published known-answer vectors of Salmon et al. (Random123)."""
import os
import subprocess
import tempfile

KATS = [
    ((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
    ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
    ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
     (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
]

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_device_header_kats():
    src = r'''
#include <stdio.h>
#include "philox.cuh"
int main(){ unsigned v[3][6] = {%s}; for (int t=0;t<3;++t){ uint32_t c[4]={v[t][0],v[t][1],v[t][2],v[t][3]};
 phx_4x32_10(c, v[t][4], v[t][5]); printf("%%08x %%08x %%08x %%08x\n", c[0],c[1],c[2],c[3]); } return 0; }
''' % ",".join("{%s}" % ",".join(str(x) for x in c + k) for c, k, _ in KATS)
    with tempfile.TemporaryDirectory() as td:
        c = os.path.join(td, "t.c")
        exe = os.path.join(td, "t")
        open(c, "w").write(src)
        subprocess.check_call(["gcc", "-O2", "-I", os.path.join(ROOT, "mpt_gb300", "csrc"), c, "-o", exe])
        lines = subprocess.check_output([exe], text=True).split("\n")
    for (_, _, want), line in zip(KATS, lines):
        assert tuple(int(x, 16) for x in line.split()) == want


def test_oracle_uniform_matches_header(orc):
    """The oracle's uniform stream equals the device header's (same counters)."""
    src = r'''
#include <stdio.h>
#include "philox.cuh"
int main(){ for (unsigned i=0;i<50;++i) printf("%a\n", phx_uniform(0x1234567890abcdefull, i*7919u, i, i%17u)); return 0; }
'''
    with tempfile.TemporaryDirectory() as td:
        c = os.path.join(td, "t.c")
        exe = os.path.join(td, "t")
        open(c, "w").write(src)
        subprocess.check_call(["gcc", "-O2", "-I", os.path.join(ROOT, "mpt_gb300", "csrc"), c, "-o", exe])
        got = [float.fromhex(x) for x in subprocess.check_output([exe], text=True).split()]
    want = [orc.uniform(0x1234567890abcdef, i * 7919, i, i % 17) for i in range(50)]
    assert got == want
    assert all(0.0 <= u < 1.0 for u in got)


def test_sample_stream_meets_the_reference_sampler_tests(orc):
    """The planners' sample stream (the oracle's restatement of the device
    sampler) against the reference's sampler tests: unit quaternions within
    4 eps (test/uniform_sampler_so3_test.cpp:42-59; 250,000 draws here), L2
    samples inside their box (test/uniform_sampler_lp_test.cpp:41-60), SO(2)
    angles in [-pi, pi) (impl/uniform_sampler_so2.hpp:57-64)."""
    import numpy as np
    eps = np.finfo(np.float64).eps
    q = orc.sample_states(orc.make_space(orc.SO3, 4), 7, [-1] * 4, [1] * 4, 250000)
    assert (np.abs((q * q).sum(axis=1) - 1.0) < 4 * eps).all()
    se3 = orc.sample_states(orc.make_space(orc.SE3, 7, (2.0, 1.0)), 8, [-1, -1, -1, -1, 1, 2, 3],
                            [1, 1, 1, 1, 4, 6, 8], 20000)
    assert (np.abs((se3[:, :4] ** 2).sum(axis=1) - 1.0) < 4 * eps).all()
    assert ((se3[:, 4:] >= [1, 2, 3]) & (se3[:, 4:] <= [4, 6, 8])).all()
    lp = orc.sample_states(orc.make_space(orc.L2, 3), 9, [1, 2, 3], [4, 6, 8], 20000)
    assert ((lp >= [1, 2, 3]) & (lp <= [4, 6, 8])).all()
    so2 = orc.sample_states(orc.make_space(orc.SO2, 10), 10, [-np.pi] * 10, [np.pi] * 10, 20000)
    assert ((so2 >= -np.pi) & (so2 < np.pi)).all()
