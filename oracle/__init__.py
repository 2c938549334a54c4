"""CPU oracle of the reweighting path -- test infrastructure only."""
