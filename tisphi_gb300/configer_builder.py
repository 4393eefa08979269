"""Scene-file loader with the reference's accessor names.

Mirrors ``SimConfiger`` of the reference (eng/configer_builder.py:3-37): a scene JSON
holds a ``Configuration`` dict, a ``Materials`` list, a ``Blocks`` list and optional
``Bodies`` / ``Motions`` lists.  ``get_cfg(name)`` reads ``Configuration[name]``
(eng/configer_builder.py:11-14); the list getters return ``[]`` when the key is absent
(eng/configer_builder.py:16-37).

Besides a path, the loader also accepts an in-memory dict, so that benchmarks and tests
can build scenes without writing files.  Keys that the reference does not know
(``jitter``, ``seed``, ``precision``) are extensions read with ``get_cfg_opt``.
"""
import copy
import json


class SimConfiger:
    def __init__(self, scene_file_path=None, config=None) -> None:
        if config is not None:
            self.config = copy.deepcopy(config)
        else:
            with open(scene_file_path, "r") as f:
                self.config = json.load(f)

    def get_cfg(self, name, enforce_exist=False):
        if enforce_exist:
            assert name in self.config["Configuration"]
        return self.config["Configuration"][name]

    def get_cfg_opt(self, name, default=None):
        """Read an optional Configuration key (extension keys have defaults)."""
        return self.config["Configuration"].get(name, default)

    def get_materials(self):
        return self.config.get("Materials", [])

    def get_blocks(self):
        return self.config.get("Blocks", [])

    def get_bodies(self):
        return self.config.get("Bodies", [])

    def get_motions(self):
        return self.config.get("Motions", [])
