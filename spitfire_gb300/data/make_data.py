"""Regenerate the bundled mechanism data (spitfire_gb300/data/*.json) from Cantera YAML mechanism files.

Each JSON file holds the ``mech_data`` dictionary that ChemicalMechanismSpec builds from a YAML file (the same
structure Spitfire pickles, mechanism.py:108-115), so a mechanism can be rebuilt where the YAML sources are not
available: ``ChemicalMechanismSpec.from_json(path)``. Run where the mechanism files exist:

    python spitfire_gb300/data/make_data.py <directory with the YAML files>
"""
import glob
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from spitfire_gb300.mechanism import ChemicalMechanismSpec  # noqa: E402

# (yaml file relative to the source directory, phase, output name)
MECHANISMS = [('h2-burke.yaml', 'h2-burke', 'h2-burke'),
              ('methane-gri30.yaml', 'methane-gri30', 'methane-gri30'),
              ('reaction_test_mechanism.yaml', None, 'reaction-test')]


def convert(src_dir):
    todo = list(MECHANISMS)
    for f in sorted(glob.glob(os.path.join(src_dir, 'old_xmls', '*.yaml'))):
        base = os.path.basename(f)[:-5]
        if 'nasa9' in base or 'const_cp' in base:
            continue
        todo.append((os.path.join('old_xmls', base + '.yaml'), None, 'unit-' + base))
    for rel, phase, name in todo:
        spec = ChemicalMechanismSpec(cantera_input=os.path.join(src_dir, rel), group_name=phase) if phase else \
            ChemicalMechanismSpec(cantera_input=os.path.join(src_dir, rel))
        with open(os.path.join(HERE, name + '.json'), 'w') as fo:
            json.dump(spec.mech_data_json(), fo, separators=(',', ':'))
        print(name, spec.n_species, spec.n_reactions)


if __name__ == '__main__':
    if len(sys.argv) != 2:
        sys.exit('usage: python -m spitfire_gb300.data.make_data <reference checkout>/tests/test_mechanisms')
    convert(sys.argv[1])
