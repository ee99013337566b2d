set output "hist_group2_MOTIF00001.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-46.2174:11.2821]
set yrange [0:125836]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_group2_MOTIF00001.dat" using 1:2 title 'MOTIF00001 (group2)' with boxes
