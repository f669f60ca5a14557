"""Genome helpers for evolutionary models (reference ``xentica/tools/genetics.py``)."""
from xentica_gb300 import core
from xentica_gb300.tools import xmath


def genome_crossover(state, num_genes, *genomes, max_genes=None,
                     mutation_prob=0, rng_name="rng"):
    """Stochastic crossover of ``genomes`` into one genome.

    Starting at a random gene and walking all ``num_genes`` genes cyclically,
    each gene is copied from a randomly chosen non-empty parent; at most
    ``max_genes`` genes are set; with ``mutation_prob > 0`` each gene that some
    parent carries may also flip.  Every random draw reads
    ``state.<rng_name>.uniform`` and so advances the cell's random stream, in
    this order: one draw for the start gene, then per gene one draw for the
    parent (and one for the mutation).

    :returns: expression of the new genome.
    """
    max_genes = max_genes or num_genes
    gene_choose = core.IntegerVariable()
    new_genome = core.IntegerVariable()
    num_genomes = core.IntegerVariable()
    num_active = core.IntegerVariable()
    new_gene = core.IntegerVariable()
    rand_val = getattr(state, rng_name).uniform
    start_gene = core.IntegerVariable()
    start_gene *= 0
    start_gene += xmath.int(rand_val * num_genes) % len(genomes)
    for step in range(num_genes):
        gene_choose *= 0
        num_genomes *= 0
        gene = (step + start_gene) % num_genes
        for genome in genomes:
            gene_choose += ((genome >> gene) & 1 & (genome > 0)) << num_genomes
            num_genomes += (genome > 0)
        rand_val = getattr(state, rng_name).uniform
        winner_gene = xmath.int(rand_val * num_genomes)
        new_gene *= 0
        new_gene += ((gene_choose >> winner_gene) & 1)
        num_active += new_gene
        new_gene *= num_active <= max_genes
        is_mutated = 0
        if mutation_prob > 0:
            is_mutated = getattr(state, rng_name).uniform < mutation_prob
            is_mutated = is_mutated * (gene_choose > 0)
        new_genome += (new_gene ^ is_mutated) << gene
    return new_genome
