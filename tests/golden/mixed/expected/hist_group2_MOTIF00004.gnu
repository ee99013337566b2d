set output "hist_group2_MOTIF00004.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-77.3407:22.2443]
set yrange [0:162201]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_group2_MOTIF00004.dat" using 1:2 title 'MOTIF00004 (group2)' with boxes
