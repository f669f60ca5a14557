"""The cases of ``ref_examples.py``: name, example model, experiment, generations."""
CASES = [  # name, model, experiment, generations
    ("GameOfLifeColor", "examples.game_of_life:GameOfLifeColor", "ColorSmall", 9),
    ("ShiftingSands", "examples.shifting_sands:ShiftingSands", "SandsSmall", 7),
    ("NoiseTV", "examples.noisetv:NoiseTV", "NoiseSmall", 5),
    ("ConservedLife", "examples.conserved_life:ConservedLife", "ConservedSmall", 6),
    ("GraviCowboys", "examples.gravicowboys:GraviCowboys", "GraviSmall", 8),
    ("EvoLife6D", "examples.evolife:EvoLife6D", "EvoLife6DSmall", 3),
]
