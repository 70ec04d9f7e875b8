"""Algorithmic FP64 operation counts used for roofline reporting.

Counted by executing the CPU restatement of the arithmetic with an
operation-counting number type (every add, multiply, divide, square root and
log1p counts as one flop); a test keeps these constants equal to that count.
One Milky Way gradient (disk + halo + bulge + nucleus) is 92 flops; a step
is every new stage evaluation plus the stage combinations, solution and error
estimate (Dopri5: 6 new evaluations thanks to FSAL; Dopri8: 13).
A stream particle's step adds the progenitor's Plummer sphere to the Milky Way
(114 flops per gradient). The learned surrogate's plain FP64 direct sum adds
512 off-centre Plummer spheres (22 flops each: 11,356 per gradient).
"""

GRADIENT_FLOPS_MW = 92
STEP_FLOPS_MW = {5: 1002, 8: 2276}
STEP_FLOPS_MW_PLUMMER = {5: 1134, 8: 2562}
STEP_FLOPS_MW_SUBHALOS = {5: 68586, 8: 148708}
