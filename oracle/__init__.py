"""CPU oracle for the BLS12-377 G1 MSM: test infrastructure, never the product path.

bls12_377 -- pure-Python big-int restatement of the reference's curve math (small cases);
cpu       -- ctypes bridge to cpu_msm.c, the arkworks-style Jacobian Pippenger (checker and the
             timed CPU baseline).
"""
