"""FP64 CPU oracle for the BristolFE-v2 explicit time-marching path.

TEST INFRASTRUCTURE ONLY. Nothing in the product package imports this
directory; only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may use it, and
there only to check results or as the timed CPU baseline, never as the
thing measured or shipped.

The reference (ndtatbristol/BristolFE-v2) is a pure MATLAB toolbox and no
MATLAB or GNU Octave exists on either machine, so the reference cannot be run.
This package restates its algorithms in NumPy/SciPy FP64, one function per
reference function, each citing the reference file:line it follows.

Parity pinning: the element routines are pinned bit-for-bit-close (1e-12
relative) against golden vectors generated by evaluating the reference's own
generated element files (``code/internal/elements/fn_el_*.m``) - see
``tests/golden/make_golden.py``. The reference ships no stored solver outputs,
so the assembly and time-marching restatements are pinned by the reference's
own known-answer physics checks (amplification-matrix spectral radius,
Schmerr fluid/solid R/T coefficients, rigid-body modes, mass totals, v5 versus
v6 'vel at last half time step' agreement) rather than by stored outputs: for
those parts parity is "unpinned" against reference outputs.
"""
