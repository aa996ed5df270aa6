"""CPU oracle of viltrum's per-bin integration path -- test infrastructure, not the product."""
