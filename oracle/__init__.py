"""CPU checkers for the GPU path (test infrastructure; the product never imports this package).

* ``oracle.bindings.Oracle``    -- the C restatement in hibf_oracle.c (always buildable, also on the GPU host).
* ``oracle.bindings.Reference`` -- the reference library itself, compiled from its sources into oracle/_ref
                                   (only where the seqan/hibf source tree is present).
"""
