"""CPU oracle for the GIGA-Lens forward model + likelihood hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
module; only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline leg may use it, and there only as the checker (or, for the CPU
baseline, as the timed CPU restatement).

The oracle is a restatement, in PyTorch-CPU arithmetic of a selectable
precision (float64 for the error reference, float32 to mimic the reference's
own float32 TensorFlow CPU path), of the reference's algorithm:

* ``gigalens/simulator.py:91-125``  coordinate grid (``get_coords``)
* ``gigalens/tf/simulator.py:11-165``  simulate / lstsq_simulate
* ``gigalens/tf/profiles/mass/{epl,shear,sis,sie}.py``  deflections
* ``gigalens/tf/profiles/light/{sersic,shapelets}.py``  light profiles
* ``gigalens/tf/model.py:53-86``  ForwardProbModel likelihood and chi^2

Parity pinning: the reference itself (TensorFlow, TFP, lenstronomy) cannot be
imported here, so the oracle is pinned by known-answer tests taken from the
reference: the Sersic half-light test (``tests/test_profiles.py:14-26``), the
EPL against the reference's closed-form SIS/SIE (``tf/profiles/mass/sis.py``,
``sie.py``), the EPL power-law limit, and the reference's own demo fixture
(``assets/demo.npy`` + ``assets/psf.npy`` with the ``tf-demo.ipynb`` truth),
whose chi^2 at the truth must be ~1.  Per-pixel parity with the reference's
own TensorFlow output is therefore *unpinned*; see ``tests/test_oracle.py``.
"""
