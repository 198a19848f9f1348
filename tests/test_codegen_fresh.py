"""The committed csrc/adjoint_effects.cuh is what adjoint_codegen.py emits
today: a change to a restated effect block that was not regenerated (or a
hand edit of the generated header) fails here."""
import os

from posidonius_gb300 import adjoint_codegen


def test_generated_effect_blocks_are_fresh():
    text, _ = adjoint_codegen.generate()
    with open(adjoint_codegen.OUT) as f:
        committed = f.read()
    assert text == committed, ("csrc/adjoint_effects.cuh differs from the generator's output; run "
                               "python -m posidonius_gb300.adjoint_codegen")
    assert os.path.basename(adjoint_codegen.OUT) == "adjoint_effects.cuh"
