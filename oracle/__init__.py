"""CPU oracle for the larnd-sim-jax simulate path.  TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package, and only as the checker or as the
timed CPU baseline; the product path (``larndsim_gb300``) never imports it.

Contents
--------
``reference_np``  float32 numpy restatement of the reference's forward chain
                  (LUT and parametrised modes, FEE, hit compaction, LUT
                  template bank), each function citing the reference
                  file:line it follows.
``grad64``        float64 restatement of the LUT-mode loss with every
                  discrete decision (bins, ticks, template index, crossing
                  indices, reset masks) frozen from a float32 forward pass,
                  plus central finite differences: the pathwise gradient the
                  reference's ``jax.value_and_grad`` computes.
``losses_np``     float64 restatement of the hit-level fit losses.
``prob_loss_np``  restatement of the likelihood losses on the probabilistic
                  front end's distributions (ProbabilisticLossStrategy,
                  compute_occurrence_indices, llhd_loss) and their
                  gradients.

Parity status: PARTIALLY PINNED.  The reference is JAX and JAX is not
installable on the machines this builds on, and its LUT-mode golden outputs
were produced with a LUT that is not distributed.  What is pinned against the
reference's own committed outputs (output/jax_ref/output_*_1.npz): the
detector geometry, the drift velocity, pixel-centre coordinates, hit z from
ticks, the digitisation of a zero charge and the ADC->charge inverse (see
tests/test_oracle_golden.py).  Waveform accumulation and the self-trigger
are restated from the source and checked with closed-form known answers.
"""
