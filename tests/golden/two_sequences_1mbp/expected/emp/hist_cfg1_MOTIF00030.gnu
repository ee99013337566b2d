set output "hist_cfg1_MOTIF00030.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-47.2138:13.3292]
set yrange [0:2021]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00030.dat" using 1:2 title 'MOTIF00030 (cfg1)' with boxes
