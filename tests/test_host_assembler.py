"""SequentialAssembler input lists checked on the host before any device
work (the six form types of src/assembly/SequentialAssembler.py:20-30)."""
import numpy as np
import pytest

import nfempy_gb300 as nf


def test_form_types_match_reference():
    asm = nf.SequentialAssembler(None, None, np.zeros(3))
    assert sorted(asm.form_type_to_callable_map) == sorted(
        ["form", "bc_form", "interface_form", "bc_interface_form", "time_dependent_form", "time_dependent_bc_form"])


def test_unknown_form_type_is_refused():
    asm = nf.SequentialAssembler(None, None, np.zeros(3))
    asm.form_to_input_list = {"x": ["mortar_form", range(3), object(), None]}
    with pytest.raises(NotImplementedError):
        asm.scatter_forms()


@pytest.mark.parametrize("entry", [["form", range(3), object()],
                                   ["time_dependent_form", range(3), object(), (None, None)],
                                   ["bc_form", range(3), object(), None, 0.5]])
def test_input_list_length_is_checked(entry):
    asm = nf.SequentialAssembler(None, None, np.zeros(3))
    asm.form_to_input_list = {"x": entry}
    with pytest.raises(ValueError):
        asm.scatter_forms()
