"""Oracle: FP64 CPU restatement of ma-shm's flat-shell loop (test infrastructure only).

Parity unpinned for the time loop: the reference ships no tests, golden
vectors or stored outputs for its MATLAB solvers, and MATLAB cannot run here.
Pinned: the GLL table of gll.m, the 3D stiffness printed in
engineering_2_C3D.m and the damage_model.m example (tests/golden/); the loop
itself is cross-checked against an independent dense assembly and energy
conservation instead."""
