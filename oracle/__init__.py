"""CPU oracle for the EMPEROR radial-velocity log-posterior and its PT sampler.

TEST INFRASTRUCTURE ONLY.  Nothing in the product path (the package
``astroemperor_gb300``) imports this package.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may use
it, and then only as the checker or as the timed reference-faithful CPU path.

Contents
--------
``oracle.rv``
    FP64 numpy restatement of the per-theta functions that EMPEROR generates
    into its temporary run script (``my_model``, ``my_likelihood``,
    ``my_prior``) together with the data preprocessing of ``DataWrapper``.
``oracle.pt``
    numpy restatement of the parallel-tempering loop (affine-invariant
    stretch move, adjacent-temperature swaps, ladder adaptation) that
    EMPEROR drives through ``reddemcee.PTSampler``.
``oracle.philox``
    numpy Philox4x32-10 (Salmon et al. 2011), used to replay the exact random
    stream of the device sampler so that chains can be compared step by step.
``oracle.cpu_baseline``
    the reference-faithful CPU timing harness (one Python call per theta,
    mapped over ``multiprocessing.Pool`` as ``support/pools/01.pool`` does).

Parity pinning
--------------
The reference itself cannot run in this environment (its import chain needs
pandas, termcolor, matplotlib, and the generated script needs the third-party
``kepler`` (kepler.py 0.0.7) and ``reddemcee`` packages, none of which are
installed).  The oracle is therefore pinned against the numbers the
reference recorded in its own example notebooks for the 51 Peg data set
(``tests/01_51peg_basic.ipynb``): the reference epoch, the data-derived prior
limits and the maximum log-likelihood of the k=0 and k=1 models; see
``tests/test_oracle_pins.py``.  No single-theta known-answer vector exists in
the reference, so single-theta values are pinned only through these
end-to-end maxima.
"""
